"""Parity of the dust-only grain phases with the oracle (FP32 like the
reference): the grain opacity (source/iteration_mod.f90:194-246), setDustPDF
(source/emission_mod.f90:1921-1986), getDustT (source/update_mod.f90:3346-3453)
and the FP64 transport through grains."""
import numpy as np
import pytest

from mocassin_xray_gb300 import abi, Context, Setup

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=["q", "nk"])
def dust_deck(request, tmp_path_factory):
    """The synthetic shell with grains from efficiency ('Q') files, and the
    same shell with the reference's silicate optical constants ('nk' file,
    cross sections from the Mie series)."""
    from mocassin_xray_gb300 import DATA_DIR, configs
    deck = configs.dust_shell(tmp_path_factory.mktemp("dust") / "d", n=15, packets=40000)
    if request.param == "nk":
        nk = DATA_DIR.parent / "dustData" / "sil-dlee.nk"
        (deck.parent / "grainspecies.dat").write_text(f"1\n'{nk}' 1.0\n")
    return deck


def test_dust_phases_match_oracle(dust_deck, data_dir, oracle_lib):
    s = Setup(dust_deck, data_dir)
    T = oracle_lib.DustTables(s)
    C1 = s.n_cells + 1
    ctx = Context(0)
    ctx.load(s)
    td0, nd = s.get(abi.ARR_TDUST), s.get(abi.ARR_NDUST)
    ctx.opacity(1)
    op, sca = ctx.get(abi.ARR_OPACITY), ctx.get(abi.ARR_SCAOPAC)
    op_o, sca_o = oracle_lib.dust_opacity(T, nd, td0)
    np.testing.assert_allclose(op[:, 1:], op_o[:, 1:], rtol=1e-6)
    np.testing.assert_allclose(sca[:, 1:], sca_o[:, 1:], rtol=1e-6)
    ctx.emission(1)
    pdf = ctx.get(abi.ARR_DUSTPDF)
    pdf_o = oracle_lib.dust_pdf(T, td0)
    np.testing.assert_allclose(pdf[:, 1:], pdf_o[:, 1:], rtol=0, atol=2e-6)
    st = ctx.transport(40000, seed=9, precision=abi.PREC_FP64)
    j = ctx.get(abi.ARR_JSTE)
    jo, _, so = oracle_lib.transport(s, op, np.zeros_like(pdf), np.zeros(C1, np.float32), n=40000, seed=9,
                                     nthreads=8, sca_opac=sca, dust_pdf=pdf)
    # the same histories and the same compensated J sums as the oracle
    assert st.crossings == so.crossings and st.scatterings == so.scatterings
    np.testing.assert_array_equal(j, jo)
    ctx.normalize_j()
    jn = ctx.get(abi.ARR_JSTE)
    bs = ctx.balance()
    td = ctx.get(abi.ARR_TDUST)
    td_o, conv_o, black_o, st_o = oracle_lib.dust_t(T, jn, td0)
    assert bs.no_hit == st_o.no_hit and bs.converged == st_o.converged
    np.testing.assert_array_equal(ctx.get(abi.ARR_LG_BLACK)[1:], black_o[1:])
    np.testing.assert_allclose(td.reshape(-1, C1)[:, 1:], td_o.reshape(-1, C1)[:, 1:], rtol=1e-5)
    ctx.close()


def test_dust_iterations_accumulate_opacity(dust_deck, data_dir):
    """On a dust-only grid the reference adds the grain opacity to the
    previous iteration's (it is never reset): iteration k carries k times the
    grain opacity while no grain sublimates."""
    s = Setup(dust_deck, data_dir)
    ctx = Context(0)
    ctx.load(s)
    st1 = ctx.iterate(20000, n_iterate_mc=1, seed=3)
    op1 = ctx.get(abi.ARR_OPACITY)
    sca1 = ctx.get(abi.ARR_SCAOPAC)
    ctx.iterate(20000, n_iterate_mc=2, seed=3, counter_base=1 << 40)
    op2 = ctx.get(abi.ARR_OPACITY)
    sca2 = ctx.get(abi.ARR_SCAOPAC)
    np.testing.assert_allclose(sca2, sca1, rtol=1e-6)
    np.testing.assert_allclose(op2[:, 1:], 2.0 * op1[:, 1:], rtol=1e-5)
    assert st1.balance.cells_updated > 0
    td = ctx.get(abi.ARR_TDUST)
    assert np.all(np.isfinite(td)) and td[0, 1:].max() > 10.0
    ctx.close()
