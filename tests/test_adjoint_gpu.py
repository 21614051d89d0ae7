"""The implicit-function adjoint of the converged per-cell balance (mcx_adjoint) at a frozen J.

* The balance with Te held (mcx_balance_opts.fix_te) leaves Te untouched and equals the oracle's
  (orc_balance_fixed_te): Ne, ion fractions and heating - cooling.
* The adjoint's per-cell gradients equal the oracle's FP64 CPU gradient (ift_line_gradient) on 64
  random cells, from the same converged state and J.
* They equal the central differences of tightly converged balances (mcx_line_sensitivities with +h
  and -h) wherever those exist, for the densities and for the abundances.
* The torch.autograd.Function over it contracts the incoming gradient with them.
The balance is updateCell's (source/update_mod.f90:15-482); the objective is outputGas's forbidden-line
luminosity (source/output_mod.f90:410-432)."""
import numpy as np
import pytest

from mocassin_xray_gb300 import abi, Context, Setup

pytestmark = pytest.mark.gpu

LINES = [(8, 3, 3, 4), (8, 2, 1, 3), (7, 2, 3, 4)]   # [OIII] 5007, [OII] 3726, [NII] 6584


@pytest.fixture(scope="module")
def field(decks, data_dir):
    s = Setup(decks["lognormal_small"], data_dir)
    ctx = Context(0)
    ctx.load(s)
    ctx.opacity(1)
    ctx.emission(1)
    ctx.transport(30000, seed=21, precision=abi.PREC_FP64)
    ctx.normalize_j()
    ctx.state_save()                      # the state the balance starts from
    yield s, ctx
    ctx.close()


def _lit_cells(ctx, n, seed):
    lit = np.nonzero(ctx.get(abi.ARR_LG_BLACK)[1:] < 1)[0] + 1
    return np.sort(np.random.default_rng(seed).choice(lit, size=min(n, lit.size), replace=False))


def test_fixed_te_balance_matches_oracle(field, oracle_lib):
    s, ctx = field
    ctx.state_restore()
    ctx.balance(precision=abi.BAL_FP64, converge=True)
    te, ne, ion = ctx.get(abi.ARR_TE), ctx.get(abi.ARR_NE), ctx.get(abi.ARR_IONDEN)
    step = (te.astype(np.float64) * 1.001).astype(np.float32)
    ctx.put(abi.ARR_TE, step)
    ctx.balance(precision=abi.BAL_FP64, converge=True, fix_te=True)
    assert np.array_equal(ctx.get(abi.ARR_TE), step)
    r = ctx.get(abi.ARR_BAL_RESID)
    T = oracle_lib.BalanceTables(s)
    o_ne, o_ion, o_r, o_conv, o_black, _ = oracle_lib.balance_fixed_te(T, ctx.get(abi.ARR_JSTE), step, ne, ion,
                                                                       nthreads=8)
    lit = np.nonzero(o_black[1:] == 0)[0] + 1
    assert np.array_equal(ctx.get(abi.ARR_LG_BLACK)[lit], o_black[lit])
    np.testing.assert_allclose(ctx.get(abi.ARR_NE)[lit], o_ne[lit], rtol=1e-6)
    gi = ctx.get(abi.ARR_IONDEN).reshape(s.info.nstages, -1, s.n_cells + 1)[:, :, lit]
    oi = o_ion.reshape(s.info.nstages, -1, s.n_cells + 1)[:, :, lit]
    np.testing.assert_allclose(gi, oi, rtol=1e-5, atol=1e-12)
    # heating - cooling at the stepped Te: far from 0, and the same on both sides
    np.testing.assert_allclose(r[lit], o_r[lit], rtol=1e-6, atol=1e-9 * np.abs(o_r[lit]).max())
    assert np.median(np.abs(r[lit])) > 0


def test_adjoint_matches_oracle_gradient(field, oracle_lib):
    s, ctx = field
    ctx.state_restore()
    a = ctx.adjoint(LINES, precision=abi.BAL_FP64, h=1e-3)
    assert a["pinned_cells"] < 0.03 * s.n_cells
    # the context is left as after the converged balance: the oracle evaluates at that state
    te, ne, ion, j = (ctx.get(x) for x in (abi.ARR_TE, abi.ARR_NE, abi.ARR_IONDEN, abi.ARR_JSTE))
    cells = _lit_cells(ctx, 64, 5)
    T = oracle_lib.BalanceTables(s)
    o = oracle_lib.ift_line_gradient(s, T, j, te, ne, ion, LINES, cells, h=1e-3, nthreads=8)
    # a cell whose converged balance found no root keeps its Te (dTe/dHden = 0): the partial
    # derivative with Te held is its gradient; a cell without a converged balance has none (0)
    held = a["dte_dhden"][cells] == 0.0
    nosol = ctx.get(abi.ARR_N_ITER_T)[cells] >= 64
    assert held.sum() <= 2 and a["no_solution_cells"] == np.count_nonzero(ctx.get(abi.ARR_N_ITER_T) >= 64)
    ok = ~held
    np.testing.assert_allclose(a["dte_dhden"][cells][ok], o["dte_dhden"][ok], rtol=1e-4,
                               atol=1e-6 * np.abs(o["dte_dhden"]).max())
    for k in range(len(LINES)):
        want = np.where(nosol, 0.0, np.where(held, o["dL_dhden_te_held"][k], o["dL_dhden"][k]))
        np.testing.assert_allclose(a["dL_dhden"][k, cells], want, rtol=1e-4, atol=1e-6 * np.abs(want).max())
    # the line sums are those of the converged balance
    lum = oracle_lib.line_cell_luminosities(s, T, te, ne, ion, cells, LINES)
    assert lum.sum() > 0


def test_adjoint_matches_central_differences(field):
    """Where the perturbed balances have a derivative (no branch crossed), the adjoint equals their
    central differences; the adjoint gives every cell with a root a value."""
    s, ctx = field
    h = 1e-3
    ctx.state_restore()
    fwd = ctx.line_sensitivities(LINES, precision=abi.BAL_FP64, h=h)
    ctx.state_restore()
    bwd = ctx.line_sensitivities(LINES, precision=abi.BAL_FP64, h=-h)
    ctx.state_restore()
    a = ctx.adjoint(LINES, precision=abi.BAL_FP64, h=h)
    np.testing.assert_allclose(a["L"], fwd["L"], rtol=1e-9)
    lit = ctx.get(abi.ARR_LG_BLACK) < 1
    lit[0] = False
    both = (fwd["dL_dhden"][0] != 0) & (bwd["dL_dhden"][0] != 0) & lit
    assert both.sum() >= 0.95 * lit.sum()
    central = 0.5 * (fwd["dL_dhden"] + bwd["dL_dhden"])
    for k in range(len(LINES)):
        scale = np.abs(central[k, both]).max()
        err = np.abs(a["dL_dhden"][k, both] - central[k, both])
        # both sides carry O(h^2) and convergence errors: below 1e-3 of the largest derivative
        # for all but a few cells
        assert np.percentile(err / scale, 99) <= 2e-3 and (err / scale).max() <= 1e-2, \
            (k, np.sort(err / scale)[-5:])
        close = err <= 1e-2 * np.abs(central[k, both]) + 1e-4 * scale
        assert close.mean() >= 0.95, (k, close.mean())
    # cells the differences leave out still get the derivative of their root
    left_out = ~both & lit
    assert np.all(np.isfinite(a["dL_dhden"][:, left_out]))
    assert np.count_nonzero(a["dL_dhden"][0, left_out]) >= \
        left_out.sum() - a["pinned_cells"] - a["no_solution_cells"]


def test_adjoint_abundance_gradient(field):
    s, ctx = field
    z = [8, 7]
    ctx.state_restore()
    fwd = ctx.line_sensitivities(LINES, abun_z=z, per_cell=False, precision=abi.BAL_FP64, h=1e-3)
    ctx.state_restore()
    bwd = ctx.line_sensitivities(LINES, abun_z=z, per_cell=False, precision=abi.BAL_FP64, h=-1e-3)
    ctx.state_restore()
    a = ctx.adjoint(LINES, abun_z=z, per_cell=False, precision=abi.BAL_FP64, h=1e-3)
    central = 0.5 * (fwd["dL_dabun"] + bwd["dL_dabun"])
    # the differences leave out the few cells that cross a branch; the adjoint keeps them
    np.testing.assert_allclose(a["dL_dabun"], central, rtol=0.02, atol=1e-3 * np.abs(central).max())


def test_adjoint_autograd(field):
    import torch
    from mocassin_xray_gb300.autograd import frozen_field_lines
    s, ctx = field
    hden0 = ctx.get(abi.ARR_HDEN)
    hden = torch.tensor(hden0.astype(np.float64), requires_grad=True)
    abun = torch.zeros(1, dtype=torch.float64, requires_grad=True)
    L = frozen_field_lines(ctx, hden, LINES, abun=abun, abun_z=[8], slot=0, precision=abi.BAL_FP64)
    w = torch.tensor([1.0, -0.5, 2.0], dtype=torch.float64)
    (w * L).sum().backward()
    ctx.state_restore()
    a = ctx.adjoint(LINES, abun_z=[8], precision=abi.BAL_FP64)
    np.testing.assert_allclose(L.detach().numpy(), a["L"], rtol=1e-12)
    np.testing.assert_allclose(hden.grad.numpy(), w.numpy() @ a["dL_dhden"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(abun.grad.numpy(), w.numpy() @ a["dL_dabun"], rtol=1e-12, atol=0)
    ctx.put(abi.ARR_HDEN, hden0)


XLINES = [(8, 3, 3, 4), (8, 2, 1, 3), (7, 2, 3, 4), (10, 3, 1, 4), (16, 2, 1, 2)]


def test_adjoint_xray_chemistry_matches_oracle(decks, data_dir, oracle_lib):
    """The X-ray chemistry (Mg, Si, Fe with inner shells and Auger electrons, 27 stages, the power-law
    source to 740 Ryd): five lines, every cell's density and three abundances against the oracle's FP64
    gradient, the densities on 64 random cells, the abundances summed over every cell."""
    s = Setup(decks["xray_small"], data_dir)
    ctx = Context(0)
    ctx.load(s)
    ctx.opacity(1)
    ctx.emission(1)
    ctx.transport(20000, seed=5, precision=abi.PREC_FP64)
    ctx.normalize_j()
    z = [8, 26, 14]
    a = ctx.adjoint(XLINES, abun_z=z, precision=abi.BAL_FP64, h=1e-3)
    te, ne, ion, j = (ctx.get(x) for x in (abi.ARR_TE, abi.ARR_NE, abi.ARR_IONDEN, abi.ARR_JSTE))
    lit = np.nonzero(ctx.get(abi.ARR_LG_BLACK)[1:] < 1)[0] + 1
    # from the deck's first J a fifth of these cells have no converged balance (their ladders do not
    # settle in 64 T-iterations): no derivative; the others are compared
    nosol = ctx.get(abi.ARR_N_ITER_T)[lit] >= 64
    ctx.close()
    assert a["no_solution_cells"] == nosol.sum() and nosol.sum() < 0.5 * lit.size
    assert np.all(a["dL_dhden"][:, lit[nosol]] == 0.0)
    lit = lit[~nosol]
    T = oracle_lib.BalanceTables(s)
    o = oracle_lib.ift_line_gradient(s, T, j, te, ne, ion, XLINES, lit, abun_z=z, h=1e-3, nthreads=8)
    held = a["dte_dhden"][lit] == 0.0
    assert a["pinned_cells"] <= held.sum() <= a["pinned_cells"] + 0.05 * lit.size
    cells = np.sort(np.random.default_rng(9).choice(lit.size, size=min(64, lit.size), replace=False))
    for k in range(len(XLINES)):
        want = np.where(held, o["dL_dhden_te_held"][k], o["dL_dhden"][k])[cells]
        np.testing.assert_allclose(a["dL_dhden"][k, lit[cells]], want, rtol=1e-4, atol=1e-6 * np.abs(want).max())
    total = np.where(held[None, None, :], o["dL_dabun_te_held"], o["dL_dabun"]).sum(axis=2)
    np.testing.assert_allclose(a["dL_dabun"], total, rtol=1e-4, atol=1e-6 * np.abs(total).max())
    assert np.all(a["L"] > 0)
