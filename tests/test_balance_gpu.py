"""Parity of the GB300 balance phase (updateCell / iterateT / ionBalance /
thermBalance / forLines+equilibrium, source/update_mod.f90 and
source/emission_mod.f90:2505-3106) with the FP64 oracle, on J computed by the
device transport and imported into the oracle.  Both run in FP64; the device's
exp/pow/log10 differ from the host's by a few ulp, so the bar is a relative
1e-6 on Te, Ne and the ionic fractions above 1e-10 (absolute 1e-16 below)."""
import numpy as np
import pytest

from mocassin_xray_gb300 import abi, Context, Setup

pytestmark = pytest.mark.gpu


def _run_j(ctx, s, n, seed):
    ctx.opacity(1)
    ctx.emission(1)
    ctx.transport(n, seed=seed, precision=abi.PREC_FP64)
    ctx.normalize_j()
    return ctx.get(abi.ARR_JSTE)


def _compare(s, oracle_lib, ctx, j, te0, ne0, ion0):
    T = oracle_lib.BalanceTables(s)
    te_o, ne_o, ion_o, conv_o, black_o, nit_o, st_o = oracle_lib.balance(T, j, te0, ne0, ion0, nthreads=8)
    st = ctx.balance()
    te, ne = ctx.get(abi.ARR_TE), ctx.get(abi.ARR_NE)
    ion = ctx.get(abi.ARR_IONDEN).reshape(-1)
    conv, black, nit = ctx.get(abi.ARR_LG_CONVERGED), ctx.get(abi.ARR_LG_BLACK), ctx.get(abi.ARR_N_ITER_T)
    assert st.no_hit == int(st_o.no_hit)
    assert np.array_equal(black[1:], black_o[1:])
    same_path = nit[1:] == nit_o[1:]
    assert same_path.mean() >= 0.99, f"T-iteration counts differ in {(~same_path).sum()} cells"
    np.testing.assert_allclose(te[1:][same_path], te_o[1:][same_path], rtol=1e-6)
    np.testing.assert_allclose(ne[1:][same_path], ne_o[1:][same_path], rtol=1e-6)
    C1 = s.n_cells + 1
    a = ion.reshape(-1, C1)[:, 1:][:, same_path]
    b = ion_o.reshape(-1, C1)[:, 1:][:, same_path]
    big = np.abs(b) > 1e-10
    np.testing.assert_allclose(a[big], b[big], rtol=1e-6)
    np.testing.assert_allclose(a[~big], b[~big], rtol=0, atol=1e-16)
    assert (conv[1:] != conv_o[1:]).sum() <= max(1, int(0.01 * s.n_cells))
    assert st.no_te_bal == pytest.approx(st_o.no_te_bal, abs=max(1, 0.01 * s.n_cells))
    return st


@pytest.mark.parametrize("name", ["h_small", "lognormal_small", "xray_small"])
def test_balance_matches_oracle(decks, data_dir, oracle_lib, name):
    s = Setup(decks[name], data_dir)
    ctx = Context(0)
    ctx.load(s)
    te0, ne0, ion0 = s.get(abi.ARR_TE), s.get(abi.ARR_NE), s.get(abi.ARR_IONDEN)
    j = _run_j(ctx, s, 30000, 5)
    st = _compare(s, oracle_lib, ctx, j, te0, ne0, ion0)
    assert st.cells_updated + st.no_hit == s.n_cells
    # TeOld / NeOld hold the pre-balance state for the next iteration's skip rule
    np.testing.assert_array_equal(ctx.get(abi.ARR_TEOLD), te0)
    ctx.close()


def test_balance_second_iteration(decks, data_dir, oracle_lib):
    """A second opacity -> emission -> transport -> balance on the updated state."""
    s = Setup(decks["lognormal_small"], data_dir)
    ctx = Context(0)
    ctx.load(s)
    _run_j(ctx, s, 30000, 7)
    ctx.balance()
    te1, ne1, ion1 = ctx.get(abi.ARR_TE), ctx.get(abi.ARR_NE), ctx.get(abi.ARR_IONDEN)
    ctx.opacity(2)
    ctx.emission(2)
    ctx.transport(30000, seed=8, precision=abi.PREC_FP64)
    ctx.normalize_j()
    j = ctx.get(abi.ARR_JSTE)
    _compare(s, oracle_lib, ctx, j, te1, ne1, ion1)
    ctx.close()


def test_emission_forbidden_lines(decks, data_dir, oracle_lib):
    """The emission phase's forLines (rec = .true.) total per cell."""
    s = Setup(decks["xray_small"], data_dir)
    ctx = Context(0)
    ctx.load(s)
    ctx.opacity(1)
    ctx.emission(1)
    fl = ctx.get(abi.ARR_FOR_LINES)
    T = oracle_lib.BalanceTables(s)
    fl_o = oracle_lib.for_lines_emission(T, s.get(abi.ARR_TE), s.get(abi.ARR_NE), s.get(abi.ARR_IONDEN))
    assert np.all(fl_o[1:] > 0)
    np.testing.assert_allclose(fl[1:], fl_o[1:], rtol=2e-6)
    ctx.close()


@pytest.mark.parametrize("name", ["lognormal_small", "xray_small"])
def test_balance_mixed_precision(decks, data_dir, oracle_lib, name):
    """The production balance (FP32 rates, collision strengths and
    exponentials; FP64 level populations, ladder and bracketing; ions below
    1e-16 per H skip the atom solve) against the FP64 oracle: Te and Ne to
    1e-4, ionic fractions above 1e-6 to 1e-3, on the cells whose T-iteration
    took the same path."""
    s = Setup(decks[name], data_dir)
    ctx = Context(0)
    ctx.load(s)
    te0, ne0, ion0 = s.get(abi.ARR_TE), s.get(abi.ARR_NE), s.get(abi.ARR_IONDEN)
    j = _run_j(ctx, s, 30000, 11)
    T = oracle_lib.BalanceTables(s)
    te_o, ne_o, ion_o, conv_o, black_o, nit_o, st_o = oracle_lib.balance(T, j, te0, ne0, ion0, nthreads=8)
    ctx.balance(precision=abi.BAL_MIXED)
    te, ne = ctx.get(abi.ARR_TE), ctx.get(abi.ARR_NE)
    ion = ctx.get(abi.ARR_IONDEN).reshape(-1)
    nit = ctx.get(abi.ARR_N_ITER_T)
    same = nit[1:] == nit_o[1:]
    assert same.mean() >= 0.98
    np.testing.assert_allclose(te[1:][same], te_o[1:][same], rtol=1e-4)
    np.testing.assert_allclose(ne[1:][same], ne_o[1:][same], rtol=1e-4)
    C1 = s.n_cells + 1
    a = ion.reshape(-1, C1)[:, 1:][:, same]
    b = ion_o.reshape(-1, C1)[:, 1:][:, same]
    big = b > 1e-6
    np.testing.assert_allclose(a[big], b[big], rtol=1e-3)
    ctx.close()


@pytest.mark.parametrize("name", ["lognormal_small", "xray_small"])
def test_cooling_surfaces_match_atom_solves(decks, data_dir, name):
    """The mixed balance reading each ion's line cooling from its cooling surface (ln G over ln Te, ln Ne,
    4-point Lagrange) against the same balance solving every ion's levels per cell and T-iteration: Te and
    Ne to 2e-5, ionic fractions above 1e-6 to 2e-4, on the cells whose T-iteration took the same path."""
    s = Setup(decks[name], data_dir)
    ctx = Context(0)
    ctx.load(s)
    _run_j(ctx, s, 30000, 11)
    ctx.state_save()
    ctx.balance(precision=abi.BAL_MIXED, atom_solves=True)
    te_a, ne_a = ctx.get(abi.ARR_TE), ctx.get(abi.ARR_NE)
    ion_a, nit_a = ctx.get(abi.ARR_IONDEN), ctx.get(abi.ARR_N_ITER_T)
    ctx.state_restore()
    ctx.balance(precision=abi.BAL_MIXED)
    te, ne = ctx.get(abi.ARR_TE), ctx.get(abi.ARR_NE)
    ion, nit = ctx.get(abi.ARR_IONDEN), ctx.get(abi.ARR_N_ITER_T)
    same = nit[1:] == nit_a[1:]
    assert same.mean() >= 0.98
    np.testing.assert_allclose(te[1:][same], te_a[1:][same], rtol=2e-5)
    np.testing.assert_allclose(ne[1:][same], ne_a[1:][same], rtol=2e-5)
    C1 = s.n_cells + 1
    a = ion.reshape(-1, C1)[:, 1:][:, same]
    b = ion_a.reshape(-1, C1)[:, 1:][:, same]
    big = b > 1e-6
    np.testing.assert_allclose(a[big], b[big], rtol=2e-4)
    ctx.close()


def test_emission_forbidden_lines_mixed(decks, data_dir, oracle_lib):
    s = Setup(decks["xray_small"], data_dir)
    ctx = Context(0)
    ctx.load(s)
    ctx.opacity(1)
    ctx.emission(1, precision=abi.PHASE_MIXED)
    fl = ctx.get(abi.ARR_FOR_LINES)
    T = oracle_lib.BalanceTables(s)
    fl_o = oracle_lib.for_lines_emission(T, s.get(abi.ARR_TE), s.get(abi.ARR_NE), s.get(abi.ARR_IONDEN))
    np.testing.assert_allclose(fl[1:], fl_o[1:], rtol=1e-4)
    ctx.close()


def test_state_save_restore(decks, data_dir):
    s = Setup(decks["h_small"], data_dir)
    ctx = Context(0)
    ctx.load(s)
    ctx.state_save()
    te0 = ctx.get(abi.ARR_TE)
    _run_j(ctx, s, 5000, 3)
    ctx.balance()
    assert not np.array_equal(ctx.get(abi.ARR_TE), te0)
    ctx.state_restore()
    np.testing.assert_array_equal(ctx.get(abi.ARR_TE), te0)
    ctx.close()
