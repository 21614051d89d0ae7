"""The oracle's implicit-function adjoint of the converged balance (ift_line_gradient) against finite
differences of the balance's root itself, all on the CPU: at fixed J each cell's converged Te is the
root of heating - cooling of the ladder converged at that Te (orc_balance_fixed_te), found here by a
secant iteration for the unperturbed and the perturbed densities and abundances; the central
differences of the line luminosities at those roots equal the adjoint's gradient.  The balance
restated is updateCell's (source/update_mod.f90:15-482); the objective is outputGas's forbidden-line
luminosity of each cell (source/output_mod.f90:410-432)."""
import numpy as np
import pytest

from mocassin_xray_gb300 import abi, configs, Setup

LINES = [(8, 3, 3, 4), (8, 2, 1, 3), (7, 2, 3, 4)]   # [OIII] 5007, [OII] 3726, [NII] 6584
H = 1e-3


def _roots(oracle_lib, T, j, te, ne, ion, cells, hden=None, abun=None, iters=40):
    """Te of every listed cell where heating = cooling, each ladder converged at its Te; returns the
    state at the roots and a mask of the cells whose iteration settled on a sign change."""
    te = te.astype(np.float32).copy()
    ne1, ion1, r1, _, _, _ = oracle_lib.balance_fixed_te(T, j, te, ne, ion, hden=hden, abun=abun, nthreads=4)
    t0, r0 = te.astype(np.float64), r1.copy()
    t1 = t0 * (1.0 + 2e-3)
    done = np.zeros(te.size, bool)
    for _ in range(iters):
        te = t1.astype(np.float32)
        ne1, ion1, r1, _, _, _ = oracle_lib.balance_fixed_te(T, j, te, ne1, ion1, hden=hden, abun=abun, nthreads=4)
        t1 = te.astype(np.float64)
        with np.errstate(divide="ignore", invalid="ignore"):
            t2 = t1 - r1 * (t1 - t0) / (r1 - r0)
        t2 = np.where(np.isfinite(t2), np.clip(t2, 0.8 * t1, 1.25 * t1), t1)
        done = np.abs(t2 - t1) <= 2e-7 * t1
        if done[cells].all():
            break
        t0, r0, t1 = t1, r1, np.where(done, t1, t2)
    return te, ne1, ion1, done


@pytest.fixture(scope="module")
def converged(tmp_path_factory, oracle_lib, data_dir):
    s = Setup(configs.lognormal_gas(tmp_path_factory.mktemp("adj") / "ln", n=7, packets=4000, half_width=2.6e18),
              data_dir)
    T = oracle_lib.BalanceTables(s)
    te0, ne0, ion0 = s.get(abi.ARR_TE), s.get(abi.ARR_NE), s.get(abi.ARR_IONDEN)
    op = oracle_lib.opacity(s)
    rec, tl = oracle_lib.emission(s, 10000.0, for_lines=oracle_lib.for_lines_emission(T, te0, ne0, ion0))
    j, _, _ = oracle_lib.transport(s, op, rec, tl, n=20000, seed=3, nthreads=4)
    j *= 1e-9
    te, ne, ion, _, black, _, _ = oracle_lib.balance(T, j, te0, ne0, ion0, nthreads=4)
    lit = np.nonzero(black[1:] == 0)[0] + 1
    rng = np.random.default_rng(7)
    cells = np.sort(rng.choice(lit, size=min(16, lit.size), replace=False))
    te, ne, ion, ok = _roots(oracle_lib, T, j, te, ne, ion, cells)
    cells = cells[ok[cells]]
    assert cells.size >= 12
    return s, T, j, te, ne, ion, cells


def test_fixed_te_holds_te_and_converges_the_ladder(converged, oracle_lib):
    s, T, j, te, ne, ion, cells = converged
    ne1, ion1, r, conv, black, rounds = oracle_lib.balance_fixed_te(T, j, te, ne, ion, nthreads=4)
    assert np.all(conv[cells] == 1) and np.all(rounds[cells] >= 1)
    # at the root the residual is at the level of Te's FP32 rounding: a step of 2 ulp moves it further
    te2 = (te.astype(np.float64) * (1.0 + 2.5e-7)).astype(np.float32)
    _, _, r2, _, _, _ = oracle_lib.balance_fixed_te(T, j, te2, ne, ion, nthreads=4)
    assert np.all(np.abs(r[cells]) <= 2.0 * np.abs(r2[cells] - r[cells]) + 1e-300)


def test_ift_density_gradient_equals_root_differences(converged, oracle_lib):
    s, T, j, te, ne, ion, cells = converged
    g = oracle_lib.ift_line_gradient(s, T, j, te, ne, ion, LINES, cells, h=H)
    hden = T.k["hden"].astype(np.float64)
    lum = {}
    for sign in (1.0, -1.0):
        hd = (hden * (1.0 + sign * H)).astype(np.float32)
        t, n, x, ok = _roots(oracle_lib, T, j, te, ne, ion, cells, hden=hd)
        assert ok[cells].all()
        lum[sign] = (oracle_lib.line_cell_luminosities(s, T, t, n, x, cells, LINES, hden=hd),
                     t[cells].astype(np.float64), hd[cells].astype(np.float64))
    dh = lum[1.0][2] - lum[-1.0][2]
    fd = (lum[1.0][0] - lum[-1.0][0]) / dh
    dte = (lum[1.0][1] - lum[-1.0][1]) / dh
    np.testing.assert_allclose(g["dte_dhden"], dte, rtol=2e-2, atol=1e-3 * np.abs(dte).max())
    for k in range(len(LINES)):
        np.testing.assert_allclose(g["dL_dhden"][k], fd[k], rtol=1e-2, atol=1e-3 * np.abs(fd[k]).max())
    # the response of Te matters: holding Te would give another gradient
    assert np.abs(g["dte_dhden"]).max() > 0


def test_ift_abundance_gradient_equals_root_differences(converged, oracle_lib):
    s, T, j, te, ne, ion, cells = converged
    z = 8
    g = oracle_lib.ift_line_gradient(s, T, j, te, ne, ion, LINES[:1], cells, abun_z=[z], h=H)
    abun = T.k["abun"].astype(np.float64)
    lum = {}
    for sign in (1.0, -1.0):
        ab = abun.astype(np.float32).copy()
        ab[z - 1] = np.float32(abun[z - 1] * (1.0 + sign * H))
        t, n, x, ok = _roots(oracle_lib, T, j, te, ne, ion, cells, abun=ab)
        assert ok[cells].all()
        lum[sign] = (oracle_lib.line_cell_luminosities(s, T, t, n, x, cells, LINES[:1], abun=ab), float(ab[z - 1]))
    fd = (lum[1.0][0] - lum[-1.0][0]) / (lum[1.0][1] - lum[-1.0][1])
    np.testing.assert_allclose(g["dL_dabun"][:, 0, :], fd, rtol=1e-2, atol=1e-3 * np.abs(fd).max())


def test_ift_xray_chemistry_equals_root_differences(tmp_path, oracle_lib, data_dir):
    """The same on the X-ray chemistry (Mg, Si, Fe with inner shells and Auger electrons, 27 stages):
    J is kept only in a dozen cells, so that the balances run on those alone."""
    s = Setup(configs.xray_gas(tmp_path / "xr", n=7, packets=4000), data_dir)
    T = oracle_lib.BalanceTables(s)
    te0, ne0, ion0 = s.get(abi.ARR_TE), s.get(abi.ARR_NE), s.get(abi.ARR_IONDEN)
    op = oracle_lib.opacity(s)
    rec, tl = oracle_lib.emission(s, 10000.0, for_lines=oracle_lib.for_lines_emission(T, te0, ne0, ion0))
    j, _, _ = oracle_lib.transport(s, op, rec, tl, n=20000, seed=3, nthreads=4)
    j *= 1e-9
    lit = np.nonzero(j.sum(axis=0)[1:] > 0)[0] + 1
    cells = np.sort(np.random.default_rng(3).choice(lit, size=min(12, lit.size), replace=False))
    keep = np.zeros(j.shape[1], bool)
    keep[cells] = True
    j = np.where(keep[None, :], j, 0.0)
    te, ne, ion, _, _, _, _ = oracle_lib.balance(T, j, te0, ne0, ion0, nthreads=4)
    te, ne, ion, ok = _roots(oracle_lib, T, j, te, ne, ion, cells)
    cells = cells[ok[cells]]
    assert cells.size >= 6
    lines = [(8, 3, 3, 4), (10, 3, 1, 4)]
    g = oracle_lib.ift_line_gradient(s, T, j, te, ne, ion, lines, cells, abun_z=[26], h=H)
    hden = T.k["hden"].astype(np.float64)
    lum = {}
    for sign in (1.0, -1.0):
        hd = (hden * (1.0 + sign * H)).astype(np.float32)
        t, n, x, ok2 = _roots(oracle_lib, T, j, te, ne, ion, cells, hden=hd)
        assert ok2[cells].all()
        lum[sign] = (oracle_lib.line_cell_luminosities(s, T, t, n, x, cells, lines, hden=hd),
                     hd[cells].astype(np.float64))
    fd = (lum[1.0][0] - lum[-1.0][0]) / (lum[1.0][1] - lum[-1.0][1])
    for k in range(len(lines)):
        assert np.count_nonzero(fd[k]) >= cells.size // 2
        np.testing.assert_allclose(g["dL_dhden"][k], fd[k], rtol=1e-2, atol=1e-3 * np.abs(fd[k]).max())
    assert np.all(np.isfinite(g["dL_dabun"])) and np.abs(g["dte_dhden"]).max() > 0
