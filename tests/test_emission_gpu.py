"""Parity of the GB300 emission kernel (re-emission CDF and line fraction) with
the FP64 oracle restatement of emissionDriver / fb_ff / twoPhoton /
RecLinesEmission / setDiffusePDF (source/emission_mod.f90).  The kernel keeps
the reference's FP32 partial sums; tolerances: 3e-5 absolute on CDF values,
3e-5 relative on the line fraction."""
import numpy as np
import pytest

from mocassin_xray_gb300 import abi, Context, Setup

pytestmark = pytest.mark.gpu


def _state(s, seed):
    rng = np.random.default_rng(seed)
    C1 = s.n_cells + 1
    te = s.get(abi.ARR_TE).copy()
    te[1:] = 5000.0 + 15000.0 * rng.random(C1 - 1)
    ne = (s.get(abi.ARR_NE) * (0.3 + rng.random(C1))).astype(np.float32)
    ion = s.get(abi.ARR_IONDEN).reshape(s.info.nstages, max(s.info.n_elem_used, 1), C1).copy()
    r = rng.random(ion.shape).astype(np.float32) ** 3
    ion = (r / r.sum(axis=0, keepdims=True)).astype(np.float32)
    return te.astype(np.float32), ne, ion


@pytest.mark.parametrize("name", ["h_small", "lognormal_small", "xray_small"])
@pytest.mark.parametrize("perturb", [False, True])
def test_emission_matches_oracle(decks, data_dir, oracle_lib, name, perturb):
    s = Setup(decks[name], data_dir)
    ctx = Context(0)
    ctx.load(s)
    if perturb:
        te, ne, ion = _state(s, 3)
        ctx.put(abi.ARR_TE, te); ctx.put(abi.ARR_NE, ne); ctx.put(abi.ARR_IONDEN, ion)
    else:
        te, ne, ion = s.get(abi.ARR_TE), s.get(abi.ARR_NE), s.get(abi.ARR_IONDEN)
    ctx.opacity(1)
    st = ctx.emission(1)
    assert st.cells_computed == s.n_cells
    rec = ctx.get(abi.ARR_RECPDF)
    tl = ctx.get(abi.ARR_TOTAL_LINES)
    compute = np.ones(s.n_cells + 1, np.uint8); compute[0] = 0
    _, te_last = oracle_lib.gaunt_cache(s.info.nx, s.info.ny, s.info.nz, s.get(abi.ARR_ACTIVE), te, compute, -1.0)
    fl = oracle_lib.for_lines_emission(oracle_lib.BalanceTables(s), te, ne, np.asarray(ion).reshape(-1))
    rec_o, tl_o = oracle_lib.emission(s, te_last, te=te, ne=ne, ionden=np.asarray(ion).reshape(-1), for_lines=fl)
    assert np.all(np.diff(rec[:, 1:], axis=0) >= 0.0)
    assert np.all(rec[-1, 1:] == 1.0)
    np.testing.assert_allclose(rec[:, 1:], rec_o[:, 1:], rtol=0, atol=3e-5)
    np.testing.assert_allclose(tl[1:], tl_o[1:], rtol=3e-5, atol=1e-9)
    ctx.close()


def test_emission_feeds_transport(decks, data_dir, oracle_lib):
    """opacity -> emission -> transport on the device, checked against the
    oracle transport run on the same device-computed tables (FP64 path)."""
    s = Setup(decks["lognormal_small"], data_dir)
    ctx = Context(0)
    ctx.load(s)
    ctx.opacity(1)
    ctx.emission(1)
    op, rec, tl = ctx.get(abi.ARR_OPACITY), ctx.get(abi.ARR_RECPDF), ctx.get(abi.ARR_TOTAL_LINES)
    st = ctx.transport(20000, seed=21, precision=abi.PREC_FP64)
    j = ctx.get(abi.ARR_JSTE)
    jo, eo, so = oracle_lib.transport(s, op, rec, tl, n=20000, seed=21, nthreads=4)
    # the same histories and the same compensated J sums as the oracle
    assert st.crossings == so.crossings and st.line_escapes == so.line_escapes
    np.testing.assert_array_equal(j, jo)
    ctx.close()
