"""Warm-restart files (writeGrid / resetGrid, source/grid_mod.f90:2646-2883 and :3051-3689) and the
SED writer (writeSED, source/output_mod.f90:2947-3064) on the host."""
import numpy as np
import pytest

from mocassin_xray_gb300 import abi, output, restart, Setup


def _state(s, seed=0):
    rng = np.random.default_rng(seed)
    C1 = s.info.n_cells + 1
    st = dict(te=s.get(abi.ARR_TE) * rng.uniform(0.5, 1.5, C1).astype(np.float32),
              ne=s.get(abi.ARR_NE) * rng.uniform(0.5, 1.5, C1).astype(np.float32),
              hden=s.get(abi.ARR_HDEN), ionden=rng.random(s.get(abi.ARR_IONDEN).size).astype(np.float32),
              converged=rng.integers(0, 2, C1).astype(np.int32), black=rng.integers(0, 2, C1).astype(np.int32))
    return st


@pytest.mark.parametrize("name", ["h_small", "lognormal_small"])
def test_grid_files_round_trip(decks, data_dir, tmp_path, name):
    s = Setup(decks[name], data_dir)
    st = _state(s)
    restart.write_grid(tmp_path, s, st)
    for f in ("grid0.out", "grid1.out", "grid2.out", "grid3.out", "photoSource.out"):
        assert (tmp_path / f).exists()
    back = restart.read_grid(tmp_path, s)
    C1 = s.info.n_cells + 1
    for k in ("te", "ne", "hden", "converged", "black"):
        np.testing.assert_array_equal(back[k][1:], np.asarray(st[k])[1:], err_msg=k)
    # ionDen: the stages the reference writes (min(Z+1, nstages) per element on) come back exactly
    S, E = s.info.nstages, max(s.info.n_elem_used, 1)
    a = back["ionden"].reshape(S, E, C1)[:, :, 1:]
    b = st["ionden"].reshape(S, E, C1)[:, :, 1:]
    xref = s.get(abi.SARR_ELEM_XREF)
    for z in range(1, 31):
        if xref[z - 1] > 0:
            top = min(z + 1, S)
            np.testing.assert_array_equal(a[:top, xref[z - 1] - 1], b[:top, xref[z - 1] - 1])
    lines = (tmp_path / "grid0.out").read_text().splitlines()
    assert lines[1].split()[:4] == [str(s.info.nx), str(s.info.ny), str(s.info.nz), str(s.info.n_cells)]


def test_reads_fortran_list_directed_output(decks, data_dir, tmp_path):
    """grid1.out as gfortran's list-directed WRITE prints it (E and D exponents, wide columns)."""
    s = Setup(decks["h_small"], data_dir)
    st = _state(s, 1)
    restart.write_grid(tmp_path, s, st)
    rows = (tmp_path / "grid1.out").read_text().splitlines()
    fort = []
    for k, r in enumerate(rows):
        te, ne, hd = (float(x) for x in r.split())
        fmt = "D" if k % 2 else "E"
        fort.append(f"   {te:15.8E}   {ne:15.8E}   {hd:15.8E}".replace("E", fmt))
    (tmp_path / "grid1.out").write_text("\n".join(fort) + "\n")
    back = restart.read_grid(tmp_path, s)
    np.testing.assert_allclose(back["te"][1:], st["te"][1:], rtol=1e-8)


def test_mismatched_grid_is_rejected(decks, data_dir, tmp_path):
    s = Setup(decks["h_small"], data_dir)
    restart.write_grid(tmp_path, s, _state(s))
    other = Setup(decks["lognormal_small"], data_dir)
    with pytest.raises(ValueError, match="grid"):
        restart.read_grid(tmp_path, other)


def test_sed_writer(decks, data_dir, tmp_path):
    s = Setup(decks["h_small"], data_dir)
    nb, C1 = s.info.nbins, s.info.n_cells + 1
    rng = np.random.default_rng(3)
    esc = rng.random((nb + 1, C1))
    total = output.write_sed(tmp_path / "SED.out", s, esc)
    assert total == pytest.approx(8.0 * esc[1:].sum(), rel=1e-12)     # symmetricXYZ deck
    rows = [l.split() for l in (tmp_path / "SED.out").read_text().splitlines()[4:4 + nb]]
    nu, wid = s.get(abi.ARR_NU), s.get(abi.ARR_WIDFLX)
    f = 10
    assert float(rows[f][0]) == pytest.approx(nu[f], rel=1e-6)
    assert float(rows[f][1]) == pytest.approx(2.9979250e10 / (nu[f] * 3.28984e15) * 1e4, rel=1e-6)
    assert float(rows[f][2]) == pytest.approx(8.0 * esc[f + 1].sum() * nu[f] / wid[f], rel=1e-6)
