"""The reference's own benchmark decks (benchmarks/gas) read by the deck grammar of libmcx, when a
MOCASSIN source tree is named by MCX_REFERENCE_DIR on the machine running the tests: the
photoionisation benchmarks parse into grids of the expected shape, and the decks that select paths
outside this library (plane-parallel illumination) are rejected with a message, not misread."""
import os
import shutil
from pathlib import Path

import pytest

from mocassin_xray_gb300 import abi, Setup

# the root of a MOCASSIN source tree, when one is on the machine
REF = os.environ.get("MCX_REFERENCE_DIR", "")
BENCH = Path(REF) / "benchmarks" / "gas"
pytestmark = pytest.mark.skipif(not REF or not BENCH.is_dir(),
                                reason="no MOCASSIN tree (MCX_REFERENCE_DIR) with its benchmark decks on this machine")


def _deck(tmp_path, name):
    src = BENCH / name / "input"
    if not src.is_dir():
        pytest.skip(f"{name} is not in the reference tree")
    shutil.copytree(src, tmp_path / "input")
    return tmp_path / "input" / "input.in"


@pytest.mark.parametrize("name,nbins", [("HII20", 600), ("HII40", 600), ("PN150", 700), ("PN75", 700)])
def test_photoionisation_benchmarks_parse(tmp_path, data_dir, name, nbins):
    s = Setup(_deck(tmp_path, name), data_dir)
    i = s.info
    assert (i.nx, i.ny, i.nz) == (13, 13, 13)
    assert i.symmetric_xyz and i.lg_gas and not i.lg_dust
    assert i.nbins == nbins and i.n_cells > 1000
    # the initial state of an ionised nebula: H mostly ionised is not assumed, X(H0) starts at 1e-5
    assert s.get(abi.ARR_TE)[1] > 0


@pytest.mark.parametrize("name", ["NLR", "X1"])
def test_plane_parallel_decks_are_rejected(tmp_path, data_dir, name):
    with pytest.raises(RuntimeError):
        Setup(_deck(tmp_path, name), data_dir)
