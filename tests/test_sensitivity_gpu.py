"""Frozen-field line sensitivities (mcx_line_sensitivities): with J fixed every cell's balance depends on
its own density only, so the all-cells-at-once density derivative equals perturbing one cell at a time;
the line sums match mcx_line_luminosities and the oracle."""
import numpy as np
import pytest

from mocassin_xray_gb300 import abi, Context, Setup

pytestmark = pytest.mark.gpu

LINES = [(8, 3, 3, 4), (8, 2, 1, 3), (7, 2, 3, 4), (10, 3, 1, 4), (16, 2, 1, 2)]   # [OIII] [OII] [NII] [NeIII] [SII]


@pytest.fixture(scope="module")
def iterated(decks, data_dir):
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


def test_line_sums_match_line_luminosities_and_oracle(iterated, oracle_lib):
    s, ctx = iterated
    ctx.state_restore()
    r = ctx.line_sensitivities(LINES, per_cell=False, precision=abi.BAL_FP64)
    g = ctx.line_luminosities()           # the state after the unperturbed balance
    hb_raw = g["hbeta_vol"] / float(np.float32(1e-16))
    for k, (z, ion, lo, up) in enumerate(LINES):
        assert r["L"][k] > 0
        assert r["L"][k] == pytest.approx(g["forb"][z - 1, ion - 1, lo - 1, up - 1] * hb_raw, rel=1e-9)
    T = oracle_lib.BalanceTables(s)
    o = oracle_lib.line_luminosities(s, T, ctx.get(abi.ARR_TE), ctx.get(abi.ARR_NE), ctx.get(abi.ARR_IONDEN),
                                     ctx.get(abi.ARR_LG_BLACK))
    ohb = o["hbeta_vol"] / float(np.float32(1e-16))
    for k, (z, ion, lo, up) in enumerate(LINES):
        assert r["L"][k] == pytest.approx(o["forb"][z - 1, ion - 1, lo - 1, up - 1] * ohb, rel=1e-9)


def _state(ctx):
    return [(a, ctx.get(a)) for a in (abi.ARR_TE, abi.ARR_NE, abi.ARR_IONDEN)]


def _put_state(ctx, st):
    for a, v in st:
        ctx.put(a, v)


def test_density_derivative_is_local(iterated):
    """All densities perturbed at once give each cell's own derivative: the central differences of 64
    random cells, each perturbed alone by +-h under the same J and continued from the same converged
    state, equal the all-at-once ones; forward and backward differences agree."""
    s, ctx = iterated
    h = 1e-3
    ctx.state_restore()
    fwd = ctx.line_sensitivities(LINES[:2], precision=abi.BAL_FP64, h=h)
    s1 = _state(ctx)                      # the converged unperturbed balance
    ctx.state_restore()
    bwd = ctx.line_sensitivities(LINES[:2], precision=abi.BAL_FP64, h=-h)
    assert fwd["branch_cells_hden"] < 0.03 * s.n_cells and bwd["branch_cells_hden"] < 0.03 * s.n_cells
    hden0 = ctx.get(abi.ARR_HDEN)
    black = ctx.get(abi.ARR_LG_BLACK)
    rng = np.random.default_rng(64)
    cand = np.nonzero(black[1:] < 1)[0] + 1
    cells = rng.choice(cand, size=min(64, cand.size), replace=False)
    _put_state(ctx, s1)
    base = ctx.line_sensitivities(LINES[:2], per_cell=False, precision=abi.BAL_FP64)["L"]
    # cells left out of the differences (no convergence, or a discontinuity crossed) carry 0
    cells = [c for c in cells if fwd["dL_dhden"][0, c] != 0 and bwd["dL_dhden"][0, c] != 0]
    assert len(cells) >= 60
    agree = 0
    for c in cells:
        one = {}
        for sign in (1.0, -1.0):
            _put_state(ctx, s1)
            hd = hden0.copy()
            hd[c] = np.float32(float(hd[c]) * (1.0 + sign * h))
            ctx.put(abi.ARR_HDEN, hd)
            one[sign] = (ctx.line_sensitivities(LINES[:2], per_cell=False, precision=abi.BAL_FP64)["L"],
                         float(hd[c]) - float(hden0[c]))
            ctx.put(abi.ARR_HDEN, hden0)
        ok = True
        for k in range(2):
            (lp, dp), (lm, dm) = one[1.0], one[-1.0]
            central = 0.5 * ((lp[k] - base[k]) / dp + (lm[k] - base[k]) / dm)
            ref = 0.5 * (fwd["dL_dhden"][k, c] + bwd["dL_dhden"][k, c])
            scale = 1e-6 * abs(base[k]) / abs(dp)
            ok &= abs(central - ref) <= 1e-3 * abs(ref) + scale
            ok &= abs(fwd["dL_dhden"][k, c] - bwd["dL_dhden"][k, c]) <= 0.02 * abs(ref) + scale
        agree += ok
    assert agree >= len(cells) - 1


@pytest.mark.parametrize("precision", [abi.BAL_FP64, abi.BAL_MIXED])
def test_abundance_derivative(iterated, precision):
    """Differences of the tightly converged balance: the forward and backward differences of every
    line's abundance derivative agree (the reference's 2 % stopping rule makes them disagree)."""
    s, ctx = iterated
    ctx.state_restore()
    fwd = ctx.line_sensitivities(LINES, abun_z=[8, 7, 10], per_cell=False, h=1e-3, precision=precision)
    ctx.state_restore()
    bwd = ctx.line_sensitivities(LINES, abun_z=[8, 7, 10], per_cell=False, h=-1e-3, precision=precision)
    d = fwd["dL_dabun"]
    # every line answers to its own element's abundance.  The sign is not fixed: at O/H = 5e-4 more
    # oxygen cools the gas enough that [OIII] 5007 can fall, the metallicity turnover of the line
    assert np.all(np.isfinite(d))
    assert d[0, 0] != 0 and d[1, 0] != 0 and d[2, 1] != 0 and d[3, 2] != 0
    assert fwd["branch_cells_abun"] < 0.03 * 3 * s.n_cells
    np.testing.assert_allclose(d, bwd["dL_dabun"], rtol=0.03, atol=1e-3 * np.abs(d).max())


def test_tight_balance_is_a_fixed_point(iterated):
    """The tightly converged balance started again from its own result stays put (Te to 1e-6), and it
    lies within the reference's 2 % residual stop of the reference-stopped balance."""
    s, ctx = iterated
    ctx.state_restore()
    ctx.balance(precision=abi.BAL_FP64)
    te_ref = ctx.get(abi.ARR_TE)
    ctx.state_restore()
    ctx.balance(precision=abi.BAL_FP64, converge=True)
    te1, nit1 = ctx.get(abi.ARR_TE), ctx.get(abi.ARR_N_ITER_T)
    lit = ctx.get(abi.ARR_LG_BLACK)[1:] < 1
    ctx.balance(precision=abi.BAL_FP64, converge=True)
    te2 = ctx.get(abi.ARR_TE)
    ok = lit & (nit1[1:] < 64)
    assert ok.sum() >= 0.98 * lit.sum()
    stay = np.abs(te2[1:][ok] / te1[1:][ok] - 1) <= 1e-6
    assert stay.mean() >= 0.995
    assert np.median(np.abs(te1[1:][ok] / te_ref[1:][ok] - 1)) < 0.02


def test_autograd_wrapper(iterated):
    """mocassin_xray_gb300.autograd.frozen_field_lines: a torch.autograd.Function whose backward
    contracts the incoming gradient with the frozen-field derivatives; its gradient matches a
    one-cell difference of its own forward."""
    import torch
    from mocassin_xray_gb300.autograd import frozen_field_lines
    s, ctx = iterated
    hden0 = ctx.get(abi.ARR_HDEN).astype(np.float64)
    hden = torch.tensor(hden0, requires_grad=True)
    abun = torch.zeros(2, dtype=torch.float64, requires_grad=True)
    L = frozen_field_lines(ctx, hden, LINES[:2], abun=abun, abun_z=[8, 7], slot=0, precision=abi.BAL_FP64,
                           method="differences")
    w = torch.tensor([1.0, 0.5], dtype=torch.float64)
    (w * L).sum().backward()
    ctx.state_restore()
    r = ctx.line_sensitivities(LINES[:2], abun_z=[8, 7], precision=abi.BAL_FP64)
    np.testing.assert_allclose(L.detach().numpy(), r["L"], rtol=1e-12)
    np.testing.assert_allclose(hden.grad.numpy(), w.numpy() @ r["dL_dhden"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(abun.grad.numpy(), w.numpy() @ r["dL_dabun"], rtol=1e-12, atol=0)
    # a one-cell difference through the forward
    g = hden.grad.numpy()
    c = int(np.argmax(np.abs(g[1:]))) + 1
    step = np.float32(hden0[c] * 1e-3)
    hp = hden0.copy()
    hp[c] = float(np.float32(hden0[c]) + step)
    Lp = frozen_field_lines(ctx, torch.tensor(hp), LINES[:2], slot=0, precision=abi.BAL_FP64, method="differences")
    fd = float((w * (Lp - L.detach())).sum()) / float(hp[c] - np.float32(hden0[c]))
    assert fd == pytest.approx(g[c], rel=0.05)
    ctx.put(abi.ARR_HDEN, hden0.astype(np.float32))
