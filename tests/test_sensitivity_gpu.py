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


def test_density_derivative_is_local(iterated):
    s, ctx = iterated
    ctx.state_restore()
    r = ctx.line_sensitivities(LINES[:2], precision=abi.BAL_MIXED)
    hden0 = ctx.get(abi.ARR_HDEN)
    ctx.state_restore()
    base = ctx.line_sensitivities(LINES[:2], per_cell=False, precision=abi.BAL_MIXED)["L"]
    black = ctx.get(abi.ARR_LG_BLACK)
    cells = [c for c in np.linspace(1, s.info.n_cells, 40).astype(int) if black[c] < 1][:16]
    for c in cells:
        ctx.state_restore()
        hd = hden0.copy()
        hd[c] = np.float32(float(hd[c]) * (1.0 + 1e-3))
        ctx.put(abi.ARR_HDEN, hd)
        one = ctx.line_sensitivities(LINES[:2], per_cell=False, precision=abi.BAL_MIXED)["L"]
        ctx.put(abi.ARR_HDEN, hden0)
        dh = float(hd[c]) - float(hden0[c])
        for k in range(2):
            fd = (one[k] - base[k]) / dh
            assert fd == pytest.approx(r["dL_dhden"][k, c], rel=1e-6, abs=1e-9 * abs(base[k]) / dh)


def test_abundance_derivative(iterated):
    s, ctx = iterated
    ctx.state_restore()
    fwd = ctx.line_sensitivities(LINES, abun_z=[8, 7, 10], per_cell=False, h=1e-3)
    ctx.state_restore()
    bwd = ctx.line_sensitivities(LINES, abun_z=[8, 7, 10], per_cell=False, h=-1e-3)
    d = fwd["dL_dabun"]
    # every line answers to its own element's abundance.  The sign is not fixed: at O/H = 5e-4 more
    # oxygen cools the gas enough that [OIII] 5007 falls, the metallicity turnover of the line
    assert np.all(np.isfinite(d))
    assert d[0, 0] != 0 and d[1, 0] != 0 and d[2, 1] != 0 and d[3, 2] != 0
    np.testing.assert_allclose(d, bwd["dL_dabun"], rtol=0.05, atol=1e-6 * np.abs(d).max())
