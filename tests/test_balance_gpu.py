"""Parity of the GB300 balance phase (updateCell / iterateT / ionBalance /
thermBalance / forLines+equilibrium, source/update_mod.f90 and
source/emission_mod.f90:2505-3106) with the FP64 oracle, on J computed by the
device transport and imported into the oracle.  Both run in FP64 with the
same portable exp / log / log10 / pow (mcx_fmath.h) and no FMA contraction,
so every cell takes the same iterateT and ionBalance branches: Te, Ne, the
ionic fractions, the convergence flags and the T-iteration counts are
asserted on every cell, to a relative 1e-6 (in practice bit for bit)."""
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
    # every cell: the same number of T-iterations, the same flags, the same state
    assert np.array_equal(nit[1:], nit_o[1:]), f"T-iteration counts differ in {(nit[1:] != nit_o[1:]).sum()} cells"
    assert np.array_equal(conv[1:], conv_o[1:])
    np.testing.assert_allclose(te[1:], te_o[1:], rtol=1e-6)
    np.testing.assert_allclose(ne[1:], ne_o[1:], rtol=1e-6)
    C1 = s.n_cells + 1
    a = ion.reshape(-1, C1)[:, 1:]
    b = ion_o.reshape(-1, C1)[:, 1:]
    big = np.abs(b) > 1e-10
    np.testing.assert_allclose(a[big], b[big], rtol=1e-6)
    np.testing.assert_allclose(a[~big], b[~big], rtol=0, atol=1e-16)
    assert st.no_te_bal == pytest.approx(st_o.no_te_bal, abs=0.5)
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


@pytest.mark.parametrize("name", ["lognormal41", "xray41"])
def test_balance_matches_oracle_41(tmp_path, data_dir, oracle_lib, name):
    """The FP64 balance at the size of the 41^3 workloads on the reference's
    own frequency mesh (nuMax = 500 Ryd: 1311 bins, H He C N O Ne S; the X-ray
    deck, nuMax = 740 Ryd: 1333 bins, plus Mg Si Fe with 27 stages, K-shell
    ionisation and Auger yields), J from 1e6 device packets imported into the
    oracle.  The oracle balances 3000 randomly chosen cells (J zeroed in the
    others, which both sides then skip as unlit); every one must match."""
    from mocassin_xray_gb300 import configs
    deck = (configs.lognormal_gas(tmp_path / "ln41", n=41, packets=10 ** 6) if name == "lognormal41"
            else configs.xray_gas(tmp_path / "xr41", n=41, packets=10 ** 6))
    s = Setup(deck, data_dir)
    assert s.nbins == (1311 if name == "lognormal41" else 1333)
    ctx = Context(0)
    ctx.load(s)
    te0, ne0, ion0 = s.get(abi.ARR_TE), s.get(abi.ARR_NE), s.get(abi.ARR_IONDEN)
    j = _run_j(ctx, s, 10 ** 6, 5)
    keep = np.zeros(s.n_cells + 1, bool)
    keep[1 + np.random.default_rng(1).choice(s.n_cells, 3000, replace=False)] = True
    j[:, ~keep] = 0.0
    ctx.put(abi.ARR_JSTE, j)
    st = _compare(s, oracle_lib, ctx, j, te0, ne0, ion0)
    assert st.cells_updated > 2500
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


def _path_bound(te, te_ref, same, frac, rtol):
    """Cells whose T-iteration took another path than the reference run's: at
    most `frac` of the cells, each within `rtol` of the reference Te (iterateT
    stops once |heating - cooling| falls below thLimit = 2 % of the larger, so
    two runs of slightly different arithmetic may stop on either side of the
    root, a few per cent apart)."""
    other = ~same
    assert other.mean() <= frac, f"{other.sum()} cells took another path"
    if other.any():
        worst = np.max(np.abs(te[1:][other].astype(float) / te_ref[1:][other] - 1.0))
        assert worst <= rtol, f"{other.sum()} cells on another path, worst Te difference {worst:.3e}"


@pytest.mark.parametrize("name", ["lognormal_small", "xray_small"])
def test_balance_mixed_precision(decks, data_dir, oracle_lib, name):
    """The production balance (FP32 rates, collision strengths, exponentials,
    ionisation ladder and level populations; FP64 Te bracketing; line cooling
    from the cooling surfaces) against the FP64 oracle: Te and Ne to 1e-4,
    ionic fractions above 1e-6 to 1e-3, on the cells whose T-iteration took the
    same path; at most 2 % of the cells take another, each within 5 % in Te."""
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
    _path_bound(te, te_o, same, 0.02, 0.05)
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
    Ne to 2e-5, ionic fractions above 1e-6 to 2e-4, on the cells whose T-iteration took the same path; at
    most 2 % of the cells take another, each within 5 % in Te."""
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
    _path_bound(te, te_a, same, 0.02, 0.05)
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


def test_state_slots_rerun_iterations(decks, data_dir):
    """A slot holds everything an iteration hands to the next (gas state and the
    skip rule's kept opacity and CDF): rerunning iterations 2 and 3 from their
    slots reproduces them bit for bit (FP64 path: compensated J, deterministic
    phases)."""
    s = Setup(decks["lognormal_small"], data_dir)
    ctx = Context(0)
    ctx.load(s)

    def iterate(it):
        ctx.opacity(it)
        ctx.emission(it)
        ctx.transport(20000, seed=3, counter_base=it << 40, precision=abi.PREC_FP64)
        ctx.normalize_j()
        ctx.balance()
        return [ctx.get(a) for a in (abi.ARR_TE, abi.ARR_NE, abi.ARR_IONDEN, abi.ARR_OPACITY, abi.ARR_RECPDF)]

    iterate(1)
    ctx.state_save(2)
    first2 = iterate(2)
    ctx.state_save(3)
    first3 = iterate(3)
    ctx.state_restore(2)
    for a, b in zip(iterate(2), first2):
        np.testing.assert_array_equal(a, b)
    ctx.state_restore(3)
    for a, b in zip(iterate(3), first3):
        np.testing.assert_array_equal(a, b)
    with pytest.raises(abi.McxError):
        ctx.state_restore(7)
    ctx.close()
