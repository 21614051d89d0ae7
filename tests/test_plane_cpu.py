"""Plane-parallel ionisation ('planeIonization', source/set_input_mod.f90:257-262):
the slab's set-up against an independent reading of the deck (source
luminosity from the plane's photon flux, source CDF cut below nu0Add,
half-width edge cells, no radial cuts, R_out reset to the grid's extent:
source/grid_mod.f90:852, :1258, :1761-1822, :2925-2981;
source/continuum_mod.f90:472-483), and the oracle's plane source and slab
boundaries (source/photon_mod.f90:795-856, :3249-3611) on known answers."""
import math

import numpy as np
import pytest

from conftest import synthetic_recpdf
from mocassin_xray_gb300 import abi, configs, Setup


def _locate(xa, x):
    """The reference's locate (source/interpolation_mod.f90:49-106), 1-based."""
    n = len(xa)
    if x > xa[-1]:
        return n
    if x < xa[0]:
        return 0
    lo, up = 0, n + 1
    for _ in range(10000):
        if up - lo < 1:
            break
        m = (up + lo) // 2
        if xa[m - 1] == x:
            return m
        if x > xa[m - 1]:
            if lo == m:
                break
            lo = m
        else:
            up = m
    return lo


@pytest.fixture(scope="module")
def slab(tmp_path_factory, data_dir):
    deck = configs.plane_slab(tmp_path_factory.mktemp("slab") / "s", nu_max=25.0)
    return deck, Setup(deck, data_dir)


def test_slab_grid(slab):
    deck, s = slab
    i = s.info
    assert i.plane_ionization == 1 and i.symmetric_xyz == 0
    assert i.n_cells == i.nx * i.ny * i.nz          # no R_in / R_out cuts
    x, y, z = (s.get(a).astype(np.float64) for a in (abi.ARR_XAXIS, abi.ARR_YAXIS, abi.ARR_ZAXIS))
    assert i.r_out == pytest.approx(math.sqrt(x[-1] ** 2 + y[-1] ** 2 + z[-1] ** 2), rel=1e-6)

    # every axis's first and last cells are half-width: the cells tile the cuboid
    def widths(a):
        w = np.empty_like(a, dtype=np.float64)
        w[1:-1] = (a[2:] - a[:-2]) / 2.0
        w[0] = (a[1] - a[0]) / 2.0
        w[-1] = (a[-1] - a[-2]) / 2.0
        return w / 1e15

    vol = np.einsum("i,j,k->ijk", widths(x), widths(y), widths(z)).reshape(-1)   # k fastest: the cell order
    np.testing.assert_allclose(s.get(abi.ARR_VOLUME)[1:], vol, rtol=2e-6)
    assert s.get(abi.ARR_VOLUME)[1:].sum() == pytest.approx(
        (x[-1] - x[0]) * (y[-1] - y[0]) * (z[-1] - z[0]) / 1e45, rel=1e-5)


def test_slab_source(slab):
    """L* = the energy flux transferred by the plane (the spectrum scaled to the
    deck's photon flux above nu0, cut below nu0Add) times the x-z extent."""
    deck, s = slab
    i = s.info
    nu = s.get(abi.ARR_NU).astype(np.float64)
    wid = s.get(abi.ARR_WIDFLX).astype(np.float64)
    mean_field, nu0, nu0_add = 2.9979e12, 1.0, 0.56
    erg = nu ** -1.3 * np.exp(-nu / 7351.0) * np.exp(-7.353e-2 / nu)
    phot = erg / (nu * 2.1799153e-11)

    def mid_locate(v):
        k = _locate(list(nu), v)
        if 0 < k < nu.size and v > (nu[k - 1] + nu[k]) / 2:
            k += 1
        return k

    k0, ka = mid_locate(nu0), mid_locate(nu0_add)
    scale = mean_field / np.sum(phot[k0 - 1:] * wid[k0 - 1:])
    transferred = np.sum(erg[ka - 1:] * wid[ka - 1:]) * scale
    x, z = s.get(abi.ARR_XAXIS).astype(np.float64), s.get(abi.ARR_ZAXIS).astype(np.float64)
    assert i.l_star == pytest.approx(transferred / 1e36 * (x[-1] - x[0]) * (z[-1] - z[0]), rel=1e-4)
    # the source CDF starts at the bin locate() gives nu0Add
    cdf = s.get(abi.ARR_SRC_CDF)
    first = _locate(list(s.get(abi.ARR_NU)), np.float32(nu0_add))
    assert np.all(cdf[:first - 1] == 0.0) and cdf[first - 1] > 0.0 and cdf[-1] == 1.0


def test_thin_slab_known_answer(slab, oracle_lib):
    """With no opacity every transported plane packet crosses the slab along +y
    once, layer by layer, and leaves through the far face: each y-layer of
    cells collects sum(J dV) = (transported packets) x deltaE x the layer's
    thickness, whatever the packets' (x, z).  Packets born below the first
    ionisation edge (the plane emits from nu0Add = 0.56 Ryd) leave at once
    untransported, as in the reference (source/photon_mod.f90:729-739)."""
    deck, s = slab
    i = s.info
    nb, C1 = i.nbins, i.n_cells + 1
    op = np.zeros((nb, C1), np.float32)
    rec = synthetic_recpdf(s.get(abi.ARR_NU), i.n_cells)
    n = 20000
    j, esc, st = oracle_lib.transport(s, op, rec, np.zeros(C1, np.float32), n=n, seed=3, nthreads=4)
    assert st.escaped == n and st.interactions == 0 and st.error == 0
    assert st.crossings % i.ny == 0
    moved = st.crossings // i.ny
    assert 0.5 * n < moved < n          # most of the plane's energy is ionising, some is not
    lstar = float(np.float32(i.l_star))
    dE = lstar / n

    def widths(a):      # cell widths along one axis, half at both ends [1e15 cm]
        a = a.astype(np.float64)
        w = np.empty_like(a)
        w[1:-1] = (a[2:] - a[:-2]) / 2.0
        w[0], w[-1] = (a[1] - a[0]) / 2.0, (a[-1] - a[-2]) / 2.0
        return w / 1e15

    wx, wy, wz = (widths(s.get(a)) for a in (abi.ARR_XAXIS, abi.ARR_YAXIS, abi.ARR_ZAXIS))
    # the FP64 volumes the oracle deposits with (J = dl deltaE / dV)
    dV = np.einsum("i,j,k->ijk", wx, wy, wz)
    per_cell = j[:, 1:].reshape(nb, i.nx, i.ny, i.nz).sum(axis=0) * dV
    np.testing.assert_allclose(per_cell.sum(axis=(0, 2)), moved * dE * wy * 1e15, rtol=1e-9)
    # the packets start spread over the plane: every (x, z) column is crossed
    assert np.all(per_cell.sum(axis=1) > 0)
    # every packet leaves: the escape tally holds the whole source energy
    assert esc.sum() == pytest.approx(lstar, rel=1e-12)


def test_slab_reflects_at_the_sides(slab, oracle_lib):
    """Diffuse packets move in every direction; the slab's x and z faces send
    them back, so every escape is through a y face, and energy is conserved:
    escaped + (re-emitted packets lost to lines) = L*."""
    deck, s = slab
    i = s.info
    op = oracle_lib.opacity(s)
    rec = synthetic_recpdf(s.get(abi.ARR_NU), i.n_cells, seed=2)
    tl = np.full(i.n_cells + 1, 0.2, np.float32)
    n = 20000
    j, esc, st = oracle_lib.transport(s, op, rec, tl, n=n, seed=5, nthreads=4)
    assert st.error == 0
    assert st.escaped + st.line_escapes + st.trapped == n
    assert st.absorptions > 0 and st.crossings > 0


def test_tabulated_spectrum_file(tmp_path, data_dir):
    """A continuum given as a file ('rauch' format: wavelength [A], H_lambda;
    source/continuum_mod.f90:214-262) is interpolated log-log onto the mesh:
    a file that tabulates a power law H_nu ~ nu^-1.3 gives the source CDF of
    the analytic power law (cut-offs far outside the mesh)."""
    c, c_ryd = 2.9979250e10, 3.2898423e15
    lam = np.logspace(0.5, 8.5, 400)                       # [A], ascending
    nu = c / (lam * 1e-8) / c_ryd                          # [Ryd]
    h_nu = nu ** -1.3
    h_lam = 4.0 * h_nu * c / (1e-8 * lam ** 2)
    cdfs = []
    for shape in ("file", "powerlaw"):
        deck = configs.plane_slab(tmp_path / shape, nu_max=25.0)
        text = deck.read_text()
        if shape == "file":
            (deck.parent / "spec.in").write_text("".join(f"{a:.9e} {b:.9e}\n" for a, b in zip(lam, h_lam)))
            text = text.replace("contShape powerlaw 1.3 7.353e-2 7351.", "contShape 'input/spec.in'")
        else:
            text = text.replace("contShape powerlaw 1.3 7.353e-2 7351.", "contShape powerlaw 1.3 1.e-30 1.e30")
        deck.write_text(text)
        cdfs.append(Setup(deck, data_dir).get(abi.ARR_SRC_CDF))
    np.testing.assert_allclose(cdfs[0], cdfs[1], rtol=0, atol=2e-5)
