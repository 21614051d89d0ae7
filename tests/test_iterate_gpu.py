"""The MC iteration loop (iterateMC, source/iteration_mod.f90:32-1497) on the
device: one whole FP64 iteration against the oracle's chain of the same
phases, and the driver's convergence bookkeeping over several iterations."""
import numpy as np
import pytest

from mocassin_xray_gb300 import abi, Context, Setup, iterate_mc

pytestmark = pytest.mark.gpu


def test_one_iteration_chain_matches_oracle(decks, data_dir, oracle_lib):
    s = Setup(decks["lognormal_small"], data_dir)
    C1 = s.n_cells + 1
    te0, ne0, ion0 = s.get(abi.ARR_TE), s.get(abi.ARR_NE), s.get(abi.ARR_IONDEN)
    n, seed = 30000, 4
    ctx = Context(0)
    ctx.load(s)
    ctx.opacity(1)
    ctx.emission(1)
    ctx.transport(n, seed=seed, precision=abi.PREC_FP64)
    ctx.normalize_j()
    ctx.balance()
    te, nit = ctx.get(abi.ARR_TE), ctx.get(abi.ARR_N_ITER_T)
    ion = ctx.get(abi.ARR_IONDEN).reshape(-1)
    ctx.close()
    # the oracle's chain of the same phases
    T = oracle_lib.BalanceTables(s)
    comp = np.ones(C1, np.uint8)
    comp[0] = 0
    gte, te_last = oracle_lib.gaunt_cache(s.info.nx, s.info.ny, s.info.nz, s.get(abi.ARR_ACTIVE), te0, comp, -1.0)
    op = oracle_lib.opacity(s, gaunt_te=gte)
    rec, tl = oracle_lib.emission(s, te_last, for_lines=oracle_lib.for_lines_emission(T, te0, ne0, ion0))
    j, _, _ = oracle_lib.transport(s, op, rec, tl, n=n, seed=seed, nthreads=8)
    j *= 1e-9
    te_o, ne_o, ion_o, _, _, nit_o, _ = oracle_lib.balance(T, j, te0, ne0, ion0, nthreads=8)
    same = nit[1:] == nit_o[1:]
    assert same.mean() >= 0.98
    np.testing.assert_allclose(te[1:][same], te_o[1:][same], rtol=1e-5)
    a = ion.reshape(-1, C1)[:, 1:][:, same]
    b = ion_o.reshape(-1, C1)[:, 1:][:, same]
    big = b > 1e-8
    np.testing.assert_allclose(a[big], b[big], rtol=1e-3)


def test_iterate_mc_bookkeeping(decks, data_dir):
    s = Setup(decks["h_small"], data_dir)
    reps = iterate_mc(s, seed=2, n_photons=20000, max_iterations=4, min_convergence=101.0)
    assert [r.iteration for r in reps] == [1, 2, 3, 4]
    for r in reps:
        assert 0.0 <= r.conv_percent <= 100.0
        assert r.ms["transport"] > 0 and r.ms["balance"] > 0
        assert r.transport["escaped"] + r.transport["line_escapes"] > 0
    # the grid settles: the mean Te change falls between the first and the last iteration
    assert reps[-1].te_change_mean < reps[0].te_change_mean


def test_iterate_mc_stops_at_min_convergence(decks, data_dir):
    s = Setup(decks["h_small"], data_dir)
    reps = iterate_mc(s, seed=2, n_photons=20000, max_iterations=5, min_convergence=0.0)
    assert len(reps) == 1


def test_mcx_iterate_equals_phase_sequence(decks, data_dir):
    """mcx_iterate (one ABI call, balance replayed from a CUDA graph) against
    the five phase calls made one by one from the same state."""
    s = Setup(decks["lognormal_small"], data_dir)
    ctx = Context(0)
    ctx.load(s)
    ctx.state_save()
    st = ctx.iterate(20000, seed=5, transport_precision=abi.PREC_FP64, balance_precision=abi.BAL_FP64,
                     emission_precision=abi.PHASE_EXACT)
    assert st.total_ms > 0 and st.balance.cells_updated > 0
    te1, nit1 = ctx.get(abi.ARR_TE), ctx.get(abi.ARR_N_ITER_T)
    ctx.state_restore()
    ctx.opacity(1)
    ctx.emission(1)
    ctx.transport(20000, seed=5, precision=abi.PREC_FP64)
    ctx.normalize_j()
    ctx.balance(max_rounds=19)          # the direct launch path (no graph)
    ctx.state_restore()
    ctx.balance()                       # graph path, same J
    te2, nit2 = ctx.get(abi.ARR_TE), ctx.get(abi.ARR_N_ITER_T)
    same = nit1[1:] == nit2[1:]
    assert same.mean() >= 0.99
    np.testing.assert_allclose(te1[1:][same], te2[1:][same], rtol=1e-6)
    # a graph replay from the same state and J is deterministic
    ctx.state_restore()
    ctx.balance()
    np.testing.assert_array_equal(ctx.get(abi.ARR_TE), te2)
    ctx.close()
