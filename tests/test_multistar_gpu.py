"""Several ionising sources ('multiPhotoSources') on the GB300: the transport of source i uses its
luminosity, position and spectrum (energyPacketDriver(iStar, ...), source/photon_mod.f90:28-416) and
its FP64 histories equal the oracle's; an MC iteration sends nPhotons / nStars packets from each
source in turn (source/iteration_mod.f90:729-753) and J adds up over them."""
import numpy as np
import pytest

from conftest import synthetic_recpdf
from mocassin_xray_gb300 import abi, configs, Context, Setup
from test_multistar_cpu import SOURCES

pytestmark = pytest.mark.gpu

KEYS = ("crossings", "interactions", "absorptions", "scatterings", "escaped", "line_escapes", "emissions",
        "trapped")


@pytest.fixture(scope="module")
def two(tmp_path_factory, data_dir, oracle_lib):
    s = Setup(configs.multi_source(tmp_path_factory.mktemp("two") / "m", SOURCES), data_dir)
    op = oracle_lib.opacity(s)
    rec = synthetic_recpdf(s.get(abi.ARR_NU), s.n_cells, seed=6)
    tl = np.full(s.n_cells + 1, 0.2, np.float32)
    ctx = Context(0)
    ctx.load(s)
    ctx.put(abi.ARR_OPACITY, op)
    ctx.put(abi.ARR_RECPDF, rec)
    ctx.put(abi.ARR_TOTAL_LINES, tl)
    yield s, ctx, op, rec, tl
    ctx.close()


def test_each_source_fp64_matches_oracle(two, oracle_lib):
    s, ctx, op, rec, tl = two
    n, seed = 20000, 31
    for istar in (1, 2):
        jo, eo, so = oracle_lib.transport(s, op, rec, tl, n=n, seed=seed, nthreads=8, istar=istar)
        assert so.error == 0 and so.absorptions > 0
        st = ctx.transport(n, seed=seed, precision=abi.PREC_FP64, istar=istar)
        for k in KEYS:
            assert getattr(st, k) == getattr(so, k), (istar, k)
        np.testing.assert_array_equal(ctx.get(abi.ARR_JSTE), jo)
        np.testing.assert_allclose(ctx.get(abi.ARR_ESCAPED), eo, rtol=1e-12, atol=0)
    with pytest.raises(RuntimeError):
        ctx.transport(10, istar=3)


def test_sources_add_up(two, oracle_lib):
    """Source 2 after source 1 without zeroing J: J is the sum of the two sources' fields."""
    s, ctx, op, rec, tl = two
    n, seed = 20000, 17
    j1, _, _ = oracle_lib.transport(s, op, rec, tl, n=n, seed=seed, nthreads=8, istar=1)
    j2, _, _ = oracle_lib.transport(s, op, rec, tl, n=n, seed=seed, counter_base=n, nthreads=8, istar=2)
    ctx.transport(n, seed=seed, precision=abi.PREC_FP64, istar=1)
    ctx.transport(n, seed=seed, counter_base=n, precision=abi.PREC_FP64, istar=2, zero=False)
    np.testing.assert_allclose(ctx.get(abi.ARR_JSTE), j1 + j2, rtol=1e-12, atol=0)


def test_iteration_runs_every_source(two, data_dir):
    s, _, _, _, _ = two
    ctx = Context(0)
    ctx.load(s)
    st = ctx.iterate(40000, seed=3, transport_precision=abi.PREC_FP64, balance_precision=abi.BAL_FP64)
    # nPhotons / nStars packets from each source, every one ending somewhere
    tr = st.transport
    assert tr.escaped + tr.line_escapes + tr.trapped == 40000
    assert st.balance.cells_updated > 0.5 * s.n_cells
    ctx.close()


def test_python_loop_equals_the_abi_iteration(two):
    """iterate_mc's source loop (one transport per source, nPhotons / nStars each on consecutive counter
    ranges, the escape tallies zeroed before each source) gives the same iteration as mcx_iterate."""
    from mocassin_xray_gb300 import iterate_mc
    s, _, _, _, _ = two
    a = Context(0)
    a.load(s)
    rep = iterate_mc(s, a, seed=7, n_photons=15000, max_iterations=1, precision=abi.PREC_FP64,
                     min_convergence=101.0)
    assert rep[0].n_photons == 30000
    b = Context(0)
    b.load(s)
    st = b.iterate(30000, seed=7, transport_precision=abi.PREC_FP64, balance_precision=abi.BAL_FP64,
                   emission_precision=abi.PHASE_EXACT)
    assert rep[0].transport["escaped"] == st.transport.escaped
    assert rep[0].transport["emissions"] == st.transport.emissions
    np.testing.assert_array_equal(a.get(abi.ARR_JSTE), b.get(abi.ARR_JSTE))
    np.testing.assert_array_equal(a.get(abi.ARR_ESCAPED), b.get(abi.ARR_ESCAPED))
    np.testing.assert_array_equal(a.get(abi.ARR_TE), b.get(abi.ARR_TE))
    a.close()
    b.close()
