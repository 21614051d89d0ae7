"""The reference's own benchmark decks (benchmarks/gas) read by the deck grammar of libmcx, when a
MOCASSIN source tree is named by MCX_REFERENCE_DIR on the machine running the tests: the
photoionisation benchmarks parse into grids of the expected shape, the plane-parallel NLR benchmark
and X-ray benchmarks parse into their slabs, and the decks that select paths outside this library
(resonance-line transfer) are rejected with a message, not misread."""
import os
import shutil
from pathlib import Path

import numpy as np
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


def test_plane_parallel_nlr_benchmark_parses(tmp_path, data_dir):
    s = Setup(_deck(tmp_path, "NLR"), data_dir)
    i = s.info
    assert i.plane_ionization == 1 and not i.symmetric_xyz
    assert (i.nx, i.ny, i.nz) == (3, 300, 3) and i.n_cells == 2700
    assert i.l_star > 0 and i.lg_gas and not i.lg_dust
    # the slab's cells tile the cuboid of the density file
    x, y, z = (s.get(a).astype(np.float64) for a in (abi.ARR_XAXIS, abi.ARR_YAXIS, abi.ARR_ZAXIS))
    assert s.get(abi.ARR_VOLUME)[1:].astype(np.float64).sum() == pytest.approx(
        (x[-1] - x[0]) * (y[-1] - y[0]) * (z[-1] - z[0]) / 1e45, rel=1e-5)


@pytest.mark.parametrize("name,lstar_ratio", [("X1", 1.0), ("X10", 10.0)])
def test_xray_plane_benchmarks_parse(tmp_path, data_dir, name, lstar_ratio):
    """The X-ray benchmarks: plane sources with a tabulated continuum file,
    31 stages; X10's plane flux is ten times X1's."""
    s = Setup(_deck(tmp_path, name), data_dir)
    i = s.info
    assert i.plane_ionization == 1 and (i.nx, i.ny, i.nz) == (3, 30, 3) and i.nstages == 31
    cdf = s.get(abi.ARR_SRC_CDF)
    assert cdf[-1] == 1.0 and np.all(np.diff(cdf) >= 0)
    ref = Setup(_deck(tmp_path / "x1", "X1"), data_dir).info.l_star
    assert i.l_star == pytest.approx(lstar_ratio * ref, rel=1e-5)


def test_resonance_line_transfer_deck_is_rejected(tmp_path, data_dir):
    with pytest.raises(RuntimeError, match="resLinesTransfer"):
        Setup(_deck(tmp_path, "X01"), data_dir)


def test_multistar_example_parses(tmp_path, data_dir):
    """The reference's multistar example (examples/multistar): 30 sources with Starburst99 spectra at
    t = 1e6 yr, spread over an octant shell; every source gets the spectrum of its file and its cell."""
    src = Path(REF) / "examples" / "multistar" / "input"
    if not src.is_dir():
        pytest.skip("examples/multistar is not in the reference tree")
    shutil.copytree(src, tmp_path / "input")
    s = Setup(tmp_path / "input" / "input.in", data_dir)
    i = s.info
    assert i.n_stars == 30 and i.symmetric_xyz and (i.nx, i.ny, i.nz) == (52, 52, 52)
    assert i.n_photons == 1000000 // 30
    stars = s.get(abi.SARR_STARS).reshape(-1, 8)
    assert np.all(stars[:, 0] == np.float32(1000.0))
    assert np.all((stars[:, 5:8] >= 1) & (stars[:, 5:8] <= 52))
    cdfs = s.get(abi.SARR_SRC_CDFS).reshape(30, -1)
    assert np.all(cdfs[:, -1] == 1.0) and np.all(np.diff(cdfs, axis=1) >= 0)


@pytest.mark.parametrize("name", ["multigridgas", "multigridgasdust"])
def test_multigrid_examples_rejected(tmp_path, data_dir, name):
    """The reference's nested-grid examples (multiGrids) select a path outside this library: the
    set-up refuses them with a message naming the keyword, instead of misreading them."""
    src = Path(REF) / "examples" / name
    if not (src / "input.in").is_file():
        pytest.skip(f"examples/{name} is not in the reference tree")
    shutil.copytree(src, tmp_path / "input")
    with pytest.raises(RuntimeError, match="multiGrids"):
        Setup(tmp_path / "input" / "input.in", data_dir)
