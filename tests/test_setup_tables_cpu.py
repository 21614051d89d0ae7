"""The set-up tables libmcx builds (csrc/setup*.cpp) against a second,
independent construction (oracle/setup_tables.py: numpy, from the deck and
the raw data files only).  These are the tables every GPU kernel and every
oracle phase reads: the frequency mesh and bin widths, the frequency
pointers, the photoionisation cross sections at their pointers (Verner fits
from data/ph1.dat and data/ph2.dat), the Compton tables, the source CDF and
luminosity, the axes, active map, densities and cell volumes.

Tolerances: the mesh is built in single precision on both sides (the
reference's REAL), so its points agree to a few float32 ulps; the tables on
the mesh are FP64 here and FP32 in the product (as in the reference), so
they agree to the float32 rounding of their own evaluation (1e-6 relative,
1e-5 where a power of y with an exponent near -10 magnifies it, and an
absolute 1e-6 on cumulative sums of a few thousand float32 terms)."""
import math

import numpy as np
import pytest

from oracle import setup_tables as ST
from mocassin_xray_gb300 import abi, Setup


@pytest.fixture(scope="module")
def verner(data_dir):
    return ST.Verner(data_dir)


def _setups(decks, data_dir):
    for name in ("h_small", "lognormal_small", "xray_small"):
        for mode in (abi.MESH_REFERENCE, abi.MESH_LOG_EDGES):
            yield name, mode, Setup(decks[name], data_dir, mesh_mode=mode)


def test_verner_known_answers(verner):
    """Published values of the Verner et al. (1996) fits (Osterbrock & Ferland
    2006, table 2.1): H0 at 13.6 eV 6.30e-18 cm^2, He0 at 24.6 eV 7.4e-18,
    He+ at 54.4 eV 1.58e-18."""
    assert verner.xsec_mb(1, 1, 1, 13.6057) * 1e-18 == pytest.approx(6.30e-18, rel=0.01)
    assert verner.xsec_mb(2, 2, 1, 24.59) * 1e-18 == pytest.approx(7.4e-18, rel=0.03)
    assert verner.xsec_mb(2, 1, 1, 54.42) * 1e-18 == pytest.approx(1.58e-18, rel=0.02)
    # hydrogenic scaling: sigma_Z(Z^2 E) = sigma_H(E) / Z^2 for the H-like fits
    e = 30.0
    assert verner.xsec_mb(2, 1, 1, 4 * e) == pytest.approx(verner.xsec_mb(1, 1, 1, e) / 4, rel=0.02)


def test_mesh_and_pointers(decks, data_dir, verner):
    for name, mode, s in _setups(decks, data_dir):
        d = ST.read_deck(decks[name])
        nu, wid = ST.mesh(d, verner, mode, data_dir)
        got_nu, got_wid = s.get(abi.ARR_NU), s.get(abi.ARR_WIDFLX)
        assert got_nu.size == nu.size, (name, mode)
        if d.nu_max > 25.0 and mode == abi.MESH_REFERENCE:
            # fill(): every point is enlo * 10^(fildel (i - 1/2)) of its segment
            np.testing.assert_allclose(got_nu, nu, rtol=2e-6, err_msg=f"{name} mode {mode}")
            np.testing.assert_allclose(got_wid, wid, rtol=2e-6)
        else:
            # the series and ionisation edges and their +-0.0003 Ryd neighbours, exactly
            edges = [np.float32(e) for e in ST.SERIES_EDGE] + list(ST.ion_edges(d, verner))
            for e in edges:
                for v in (e, np.float32(e - np.float32(0.0003)), np.float32(e + np.float32(0.0003))):
                    if v < np.float32(d.nu_max):
                        assert v in got_nu, (name, v)
            # the log points: each follows its predecessor by one single-precision
            # step of 10^(log10(nu) + step), checked on the product's own points
            log_pts = ST.log_points(got_nu, d, verner)
            step = (np.log10(np.float64(log_pts[-1])) - np.log10(np.float64(log_pts[0]))) / (log_pts.size - 1)
            ratio = np.log10(log_pts[1:].astype(np.float64)) - np.log10(log_pts[:-1].astype(np.float64))
            np.testing.assert_allclose(ratio, step, rtol=2e-3)
            # the chained single-precision recurrence drifts by a few 1e-5 over hundreds of points
            np.testing.assert_allclose(got_nu, nu, rtol=1e-4, err_msg=f"{name} mode {mode}")
            np.testing.assert_allclose(got_wid, ST.wid_flx(got_nu), rtol=1e-6)
        ptr = s.get(abi.SARR_POINTERS)
        p = ST.pointers(nu)
        names = ["HlevNuP1", "HeIlevNuP1", "HeIIlevNuP1", "lymanP", "KshellLimitP", "secIonP", "cRecoilHP",
                 "cRecoilHeP", "xrayP", "BjumpP"]
        idx = [1, 3, 5, 7, 8, 9, 10, 11, 12, 13]
        for k, i in zip(names, idx):
            assert int(ptr[i]) == p[k], (name, mode, k, int(ptr[i]), p[k])
        np.testing.assert_allclose(s.get(abi.SARR_ION_EDGE), ST.ion_edges(d, verner), rtol=1e-7)


def test_cross_sections(decks, data_dir, verner):
    """xSecArray at its pointers: H I, He I and He II ground states, free-free,
    and every shell of every ion of the heavy elements (makeOpacity)."""
    for name, mode, s in _setups(decks, data_dir):
        d = ST.read_deck(decks[name])
        nu = s.get(abi.ARR_NU)
        xs = s.get(abi.ARR_XSEC).astype(np.float64)
        ptr = s.get(abi.SARR_POINTERS)
        p = ST.pointers(nu)
        ref = ST.xsec_h_he(verner, nu, p)
        for key, xp in (("h", 0), ("he1", 2), ("he2", 4)):
            got = xs[int(ptr[xp]) - 1: int(ptr[xp]) - 1 + ref[key].size]
            np.testing.assert_allclose(got, ref[key], rtol=1e-5, atol=1e-30, err_msg=f"{name} {key}")
        got = xs[int(ptr[6]) - 1: int(ptr[6]) - 1 + nu.size]
        np.testing.assert_allclose(got, ref["brems"], rtol=2e-6)
        nsh, ep = ST.element_p(d, verner, nu)
        got_ep = s.get(abi.SARR_ELEMENT_P).reshape(30, 30, 7, 3)
        got_nsh = s.get(abi.SARR_N_SHELLS).reshape(30, 30)
        checked = 0
        for (elem, ion), n in nsh.items():
            if ion > d.nstages:
                continue
            assert got_nsh[elem - 1, ion - 1] == n, (name, elem, ion)
            for shell in range(1, n + 1):
                p1, p2 = ep[(elem, ion, shell)]
                g1, g2, g3 = (int(v) for v in got_ep[elem - 1, ion - 1, shell - 1])
                assert (g1, g2) == (p1, p2), (name, mode, elem, ion, shell, (g1, g2), (p1, p2))
                if p2 >= p1:
                    want = ST.xsec_shell(verner, elem, ion, shell, nu, p1, p2)
                    np.testing.assert_allclose(xs[g3 - 1: g3 - 1 + want.size], want, rtol=1e-5, atol=1e-32,
                                               err_msg=f"{name} Z={elem} ion={ion} shell={shell}")
                    checked += want.size
        assert checked > 0 or not (d.abun[2:] > 1e-12).any()


def test_compton_tables(decks, data_dir):
    for name, mode, s in _setups(decks, data_dir):
        nu = s.get(abi.ARR_NU)
        c = ST.compton(nu, ST.pointers(nu)["xrayP"])
        np.testing.assert_allclose(s.get(abi.ARR_KN_SIGMA_T), c["kn_sigma_t"], rtol=2e-6)
        np.testing.assert_allclose(s.get(abi.ARR_KN_CDF).reshape(180, nu.size).T, c["kn_cdf"], rtol=0, atol=2e-6)
        np.testing.assert_allclose(s.get(abi.ARR_PCOMP).reshape(180, nu.size).T, c["pcomp"], rtol=1e-6)
        np.testing.assert_allclose(s.get(abi.SARR_COMXSEC_H), c["comxsec_h"], rtol=2e-6)
        np.testing.assert_allclose(s.get(abi.SARR_COMXSEC_C), c["comxsec_c"], rtol=2e-6)
        np.testing.assert_allclose(s.get(abi.SARR_XSEC_RECOIL), c["xsec_recoil"], rtol=1e-6)
        # small dx: the reference's formula (with (1 + 2 dx)^3 in its last term) tends to sigma_T (1 - dx / 2)
        rec = s.get(abi.SARR_XSEC_RECOIL).astype(np.float64)
        dx = nu.astype(np.float64) / 3.7573e4
        small = (np.arange(1, nu.size + 1) > ST.pointers(nu)["xrayP"]) & (dx < 0.01)
        np.testing.assert_allclose(rec[small], 6.65e-25 * (1 - dx[small] / 2), rtol=2e-4)
    # the Klein-Nishina total tends to the Thomson cross section (8 pi / 3) r_e^2 at low energy
    lo = ST.compton(np.array([1e-3], np.float32), 1)
    assert lo["kn_sigma_t"][0] == pytest.approx(8 * math.pi / 3 * 2 * 3.970393838e-26, rel=2e-4)


def test_source_spectrum(decks, data_dir):
    for name, mode, s in _setups(decks, data_dir):
        d = ST.read_deck(decks[name])
        nu, wid = s.get(abi.ARR_NU), s.get(abi.ARR_WIDFLX)
        src = ST.source(d, nu, wid)
        np.testing.assert_allclose(s.get(abi.ARR_SRC_CDF), src["cdf"], rtol=0, atol=2e-6)
        assert s.info.l_star == pytest.approx(src["l_star"], rel=2e-5), name
    # Q(H) <-> L of a blackbody in closed form: L / (4 pi R^2) = sigma T^4 and
    # Q / (4 pi R^2) = (2 pi / c^2) (kT / h)^3 int_{x0}^inf x^2 / (e^x - 1) dx,
    # x0 = h nu(1 Ryd) / kT; the reference takes Q from its mesh quadrature
    quad = pytest.importorskip("scipy.integrate").quad
    d = ST.read_deck(decks["h_small"])
    s = Setup(decks["h_small"], data_dir)
    h, k, c = 6.6262e-27, 1.380658e-16, 2.9979250e10
    t = d.t_stellar
    x0 = h * 3.2898423e15 / (k * t)
    q_per_area = 2 * math.pi / c ** 2 * (k * t / h) ** 3 * quad(lambda x: x * x / math.expm1(x), x0, 200)[0]
    l_per_q = 5.66956e-5 * t ** 4 / q_per_area
    assert s.info.l_star * 1e36 == pytest.approx(d.l_phot * 1e36 * l_per_q, rel=3e-3)


def test_grid_and_volumes(decks, data_dir):
    for name in ("h_small", "lognormal_small", "xray_small"):
        s = Setup(decks[name], data_dir)
        d = ST.read_deck(decks[name])
        g = ST.grid(d)
        np.testing.assert_array_equal(s.get(abi.ARR_XAXIS), g["x"])
        np.testing.assert_array_equal(s.get(abi.ARR_YAXIS), g["y"])
        np.testing.assert_array_equal(s.get(abi.ARR_ZAXIS), g["z"])
        act = s.get(abi.ARR_ACTIVE).reshape(d.nz, d.ny, d.nx)
        np.testing.assert_array_equal(act, g["active"].transpose(2, 1, 0))
        np.testing.assert_allclose(s.get(abi.ARR_HDEN), g["hden"], rtol=1e-7)
        vol = ST.volumes(d, g)
        np.testing.assert_allclose(s.get(abi.ARR_VOLUME)[1:], vol[1:], rtol=2e-6)
        # the volumes tile a cube: getVolume gives the edge cells of a full grid
        # a whole spacing (not half), so the cells cover (2 R + spacing)^3
        if name == "xray_small":
            side = 2 * d.edges[0] / 1e15
            assert vol[1:].sum() == pytest.approx((side * (1 + 1 / (d.nx - 1))) ** 3, rel=1e-5)
