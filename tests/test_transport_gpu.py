"""Parity of the GB300 transport kernels with the FP64 oracle.

Packet k draws from the same Philox stream in both, and the FP64 plain path
and the oracle evaluate log, cos and sin with the same portable routines
(mcx_fmath.h) and no FMA contraction, so they follow the same histories step
for step.  Both accumulate J with compensated sums (each addition's exact
rounding error kept beside it), which makes J the correctly rounded sum of
the deposits whatever their order: the FP64 J equals the oracle's entry for
entry, and the production path's J is the same bits from run to run.  The
production FP32-geometry path follows the same histories except where a
float rounding flips a discrete decision; it is checked statistically.
"""
import numpy as np
import pytest

from conftest import synthetic_recpdf
from mocassin_xray_gb300 import abi, configs, Context, Setup

pytestmark = pytest.mark.gpu


def _case(decks, data_dir, oracle_lib, name):
    s = Setup(decks[name], data_dir)
    op = oracle_lib.opacity(s)
    rec = synthetic_recpdf(s.get(abi.ARR_NU), s.n_cells)
    tl = np.full(s.n_cells + 1, 0.3, np.float32)
    ctx = Context(0)
    ctx.load(s)
    ctx.put(abi.ARR_OPACITY, op)
    ctx.put(abi.ARR_RECPDF, rec)
    ctx.put(abi.ARR_TOTAL_LINES, tl)
    return s, op, rec, tl, ctx


@pytest.mark.parametrize("name", ["h_small", "lognormal_small"])
def test_fp64_transport_matches_oracle(decks, data_dir, oracle_lib, name):
    s, op, rec, tl, ctx = _case(decks, data_dir, oracle_lib, name)
    n, seed = 20000, 1234
    st = ctx.transport(n, seed=seed, precision=abi.PREC_FP64)
    j = ctx.get(abi.ARR_JSTE)
    esc = ctx.get(abi.ARR_ESCAPED)
    jo, eo, so = oracle_lib.transport(s, op, rec, tl, n=n, seed=seed, nthreads=4)
    assert so.error == 0
    # identical histories: identical event counts
    for k in ("crossings", "interactions", "absorptions", "scatterings", "escaped", "line_escapes", "emissions",
              "trapped"):
        assert getattr(st, k) == getattr(so, k), k
    # compensated sums on both sides: every J entry is the correctly rounded sum of the same deposits
    np.testing.assert_array_equal(j, jo)
    assert esc.sum() == pytest.approx(eo.sum(), rel=1e-12)
    assert st.q_phot == pytest.approx(so.q_phot, rel=1e-12)
    ctx.close()


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_FP32_GEOM])
def test_trapped_handoff_changes_nothing(decks, data_dir, oracle_lib, precision):
    """Histories moved to the trapped-packet kernels (after 1 or 3
    re-emissions here, so that every re-emitted history moves: ~1e4 of 1e5
    packets, run one per warp, and at 8e5 packets more than 7300, run one per
    lane) give the same J bits, the same event counts and the same escapes as
    histories kept in the main kernel, also when more histories qualify than
    the 65536 the parking buffer holds (the rest stay in place); the FP64 path
    also equals the oracle."""
    s, op, rec, tl, ctx = _case(decks, data_dir, oracle_lib, "lognormal_small")
    n, seed = 100000, 4321
    ref = ctx.transport(n, seed=seed, precision=precision, handoff_emissions=-1)
    assert ref.handed_off == 0
    j0, e0 = ctx.get(abi.ARR_JSTE), ctx.get(abi.ARR_ESCAPED)
    keys = ("crossings", "interactions", "absorptions", "scatterings", "escaped", "line_escapes", "emissions", "trapped")
    for at in (1, 3):
        st = ctx.transport(n, seed=seed, precision=precision, handoff_emissions=at)
        assert st.handed_off > 0
        for k in keys:
            assert getattr(st, k) == getattr(ref, k), (at, k)
        assert st.q_phot == pytest.approx(ref.q_phot, rel=1e-12)
        np.testing.assert_array_equal(ctx.get(abi.ARR_JSTE), j0)
        np.testing.assert_allclose(ctx.get(abi.ARR_ESCAPED), e0, rtol=1e-12, atol=0)
    if precision == abi.PREC_FP64:
        jo, _, so = oracle_lib.transport(s, op, rec, tl, n=n, seed=seed, nthreads=8)
        np.testing.assert_array_equal(j0, jo)
        for k in keys:
            assert getattr(ref, k) == getattr(so, k), k
    # more qualifying histories than parking room
    big = 800000
    ref = ctx.transport(big, seed=seed, precision=precision, handoff_emissions=-1)
    j0 = ctx.get(abi.ARR_JSTE)
    st = ctx.transport(big, seed=seed, precision=precision, handoff_emissions=1)
    assert st.handed_off == 65536
    for k in keys:
        assert getattr(st, k) == getattr(ref, k), k
    np.testing.assert_array_equal(ctx.get(abi.ARR_JSTE), j0)
    ctx.close()


def test_fp32_transport_is_reproducible(decks, data_dir, oracle_lib):
    """The production path's J does not depend on the order in which the
    atomics land (scheduling, block shape): the same seed gives the same bits."""
    s, op, rec, tl, ctx = _case(decks, data_dir, oracle_lib, "lognormal_small")
    ctx.transport(30000, seed=77, precision=abi.PREC_FP32_GEOM)
    j1 = ctx.get(abi.ARR_JSTE)
    ctx.transport(30000, seed=77, precision=abi.PREC_FP32_GEOM, block_size=96, grid_mult=1)
    j2 = ctx.get(abi.ARR_JSTE)
    np.testing.assert_array_equal(j1, j2)
    ctx.close()


@pytest.mark.parametrize("name", ["h_small", "lognormal_small"])
def test_fp32_transport_statistics(decks, data_dir, oracle_lib, name):
    s, op, rec, tl, ctx = _case(decks, data_dir, oracle_lib, name)
    n, seed = 40000, 99
    st = ctx.transport(n, seed=seed, precision=abi.PREC_FP32_GEOM)
    j = ctx.get(abi.ARR_JSTE)
    esc = ctx.get(abi.ARR_ESCAPED)
    jo, eo, so = oracle_lib.transport(s, op, rec, tl, n=n, seed=seed, nthreads=4)
    # energy is conserved exactly by the bookkeeping
    de = float(np.float32(s.info.l_star)) / n
    assert esc.sum() + st.line_escapes * de == pytest.approx(float(np.float32(s.info.l_star)), rel=1e-9)
    assert st.escaped + st.line_escapes == n
    # same random integers, FP32 geometry: the histories mostly coincide
    assert st.crossings == pytest.approx(so.crossings, rel=2e-3)
    assert st.absorptions == pytest.approx(so.absorptions, rel=5e-3, abs=5)
    # J integrated over frequency per cell agrees within 1 % where the oracle's MC noise is small
    jc, joc = j[:, 1:].sum(0), jo[:, 1:].sum(0)
    hit = joc > np.percentile(joc, 50)
    assert np.median(np.abs(jc[hit] / joc[hit] - 1)) < 1e-3
    assert jc.sum() == pytest.approx(joc.sum(), rel=2e-3)
    ctx.close()


def test_transport_sharding_composes(decks, data_dir, oracle_lib):
    """Two calls over packet ranges [0,n/2) and [n/2,n) accumulate the same
    estimators as one call over [0,n) (how ranks shard packets)."""
    s, op, rec, tl, ctx = _case(decks, data_dir, oracle_lib, "h_small")
    n = 10000
    ctx.transport(n, seed=5, precision=abi.PREC_FP64)
    j_all = ctx.get(abi.ARR_JSTE)
    ctx.transport(n // 2, seed=5, precision=abi.PREC_FP64, n_photons_norm=n)
    ctx.transport(n // 2, seed=5, counter_base=n // 2, precision=abi.PREC_FP64, n_photons_norm=n, zero=False)
    j_two = ctx.get(abi.ARR_JSTE)
    # the second call adds its compensated sum to the first's rounded one: two roundings instead of one
    np.testing.assert_allclose(j_two, j_all, rtol=1e-15, atol=1e-300)
    ctx.close()


def test_normalize_j(decks, data_dir, oracle_lib):
    s, op, rec, tl, ctx = _case(decks, data_dir, oracle_lib, "h_small")
    ctx.transport(2000, seed=1, precision=abi.PREC_FP64)
    j = ctx.get(abi.ARR_JSTE)
    ctx.normalize_j()
    jn = ctx.get(abi.ARR_JSTE)
    # octant mode: (J * 1e-9) / 8  (source/iteration_mod.f90:1002-1031)
    np.testing.assert_array_equal(jn, (j * 1e-9) / 8.0)
    ctx.close()


def test_block_shapes_give_identical_results(decks, data_dir, oracle_lib):
    """Scheduling (block size, blocks per SM) does not change any history."""
    s, op, rec, tl, ctx = _case(decks, data_dir, oracle_lib, "lognormal_small")
    ctx.transport(8000, seed=2, precision=abi.PREC_FP64, block_size=256)
    j1 = ctx.get(abi.ARR_JSTE)
    ctx.transport(8000, seed=2, precision=abi.PREC_FP64, block_size=64, grid_mult=1)
    j2 = ctx.get(abi.ARR_JSTE)
    np.testing.assert_array_equal(j2, j1)
    ctx.close()


@pytest.mark.parametrize("views", ["2 0.5 1.0 2.0 5.5", "2 0.8 -1 2.2 -1"])
def test_viewing_angle_planes_match_oracle(tmp_path, data_dir, oracle_lib, views):
    """Escapes binned into the viewing-angle planes of escapedPackets
    (source/photon_mod.f90:2293-2378), FP64 path against the oracle: the
    same totals per plane (a packet on a bin boundary may land one bin over
    on either side, so to a few deltaE), plane 0 included.  The reference's
    phi = atan(vy / vx) spans (-pi/2, pi/2) only, so the views take phi bins
    it reaches (1.0 and 5.5 rad)."""
    deck = configs.lognormal_gas(tmp_path / "ln", n=13, packets=20000, half_width=1.5e19)
    deck.write_text(deck.read_text() + f"inclination {views}\n")
    s = Setup(deck, data_dir)
    op = oracle_lib.opacity(s)
    rec = synthetic_recpdf(s.get(abi.ARR_NU), s.n_cells)
    tl = np.full(s.n_cells + 1, 0.3, np.float32)
    ctx = Context(0)
    ctx.load(s)
    ctx.put(abi.ARR_OPACITY, op)
    ctx.put(abi.ARR_RECPDF, rec)
    ctx.put(abi.ARR_TOTAL_LINES, tl)
    n = 40000
    st = ctx.transport(n, seed=5, precision=abi.PREC_FP64)
    esc = ctx.get(abi.ARR_ESCAPED)
    assert esc.shape == (3, s.nbins + 1, s.n_cells + 1)
    jo, eo, so = oracle_lib.transport(s, op, rec, tl, n=n, seed=5, nthreads=4)
    de = float(np.float32(s.info.l_star)) / n
    assert st.escaped == so.escaped
    for k in range(3):
        assert esc[k].sum() == pytest.approx(eo[k].sum(), abs=4 * de), k
    assert esc[1].sum() > 0 and esc[2].sum() > 0
    ctx.close()


@pytest.fixture(scope="module")
def slab_deck(tmp_path_factory):
    return configs.plane_slab(tmp_path_factory.mktemp("slab") / "s", nu_max=25.0)


def test_plane_slab_fp64_matches_oracle(slab_deck, data_dir, oracle_lib):
    """Plane-parallel ionisation: packets born on y = 0 moving along +y, the
    slab's x and z faces reflecting, escapes through the y faces
    (source/photon_mod.f90:795-856, :3249-3611): the FP64 histories equal the
    oracle's, J bit for bit, with the hand-off to the trapped-packet kernels
    on and off."""
    s = Setup(slab_deck, data_dir)
    op = oracle_lib.opacity(s)
    rec = synthetic_recpdf(s.get(abi.ARR_NU), s.n_cells, seed=4)
    tl = np.full(s.n_cells + 1, 0.2, np.float32)
    ctx = Context(0)
    ctx.load(s)
    ctx.put(abi.ARR_OPACITY, op)
    ctx.put(abi.ARR_RECPDF, rec)
    ctx.put(abi.ARR_TOTAL_LINES, tl)
    n, seed = 30000, 71
    jo, eo, so = oracle_lib.transport(s, op, rec, tl, n=n, seed=seed, nthreads=8)
    assert so.error == 0 and so.absorptions > 0
    keys = ("crossings", "interactions", "absorptions", "scatterings", "escaped", "line_escapes", "emissions",
            "trapped")
    for at in (-1, 1):
        st = ctx.transport(n, seed=seed, precision=abi.PREC_FP64, handoff_emissions=at)
        for k in keys:
            assert getattr(st, k) == getattr(so, k), (at, k)
        np.testing.assert_array_equal(ctx.get(abi.ARR_JSTE), jo)
        np.testing.assert_allclose(ctx.get(abi.ARR_ESCAPED), eo, rtol=1e-12, atol=0)
    # the production precision moves histories between kernels without changing them either
    ref = ctx.transport(n, seed=seed, precision=abi.PREC_FP32_GEOM, handoff_emissions=-1)
    j32 = ctx.get(abi.ARR_JSTE)
    st = ctx.transport(n, seed=seed, precision=abi.PREC_FP32_GEOM, handoff_emissions=1)
    assert st.handed_off > 0 and all(getattr(st, k) == getattr(ref, k) for k in keys)
    np.testing.assert_array_equal(ctx.get(abi.ARR_JSTE), j32)
    ctx.close()


def test_plane_slab_thin_known_answer(slab_deck, data_dir):
    """No opacity: every transported packet crosses each y-layer once, so each
    layer collects sum(J dV) = transported packets x deltaE x thickness."""
    s = Setup(slab_deck, data_dir)
    i = s.info
    C1, nb = s.n_cells + 1, s.nbins
    ctx = Context(0)
    ctx.load(s)
    ctx.put(abi.ARR_OPACITY, np.zeros((nb, C1), np.float32))
    ctx.put(abi.ARR_RECPDF, synthetic_recpdf(s.get(abi.ARR_NU), s.n_cells))
    ctx.put(abi.ARR_TOTAL_LINES, np.zeros(C1, np.float32))
    n = 100000
    st = ctx.transport(n, seed=9, precision=abi.PREC_FP64)
    assert st.escaped == n and st.interactions == 0 and st.crossings % i.ny == 0
    j = ctx.get(abi.ARR_JSTE)

    def widths(a):
        a = a.astype(np.float64)
        w = np.empty_like(a)
        w[1:-1] = (a[2:] - a[:-2]) / 2.0
        w[0], w[-1] = (a[1] - a[0]) / 2.0, (a[-1] - a[-2]) / 2.0
        return w / 1e15

    wx, wy, wz = (widths(s.get(a)) for a in (abi.ARR_XAXIS, abi.ARR_YAXIS, abi.ARR_ZAXIS))
    per_cell = j[:, 1:].reshape(nb, i.nx, i.ny, i.nz).sum(axis=0) * np.einsum("i,j,k->ijk", wx, wy, wz)
    dE = float(np.float32(i.l_star)) / n
    np.testing.assert_allclose(per_cell.sum(axis=(0, 2)), (st.crossings // i.ny) * dE * wy * 1e15, rtol=1e-9)
    ctx.close()


def test_plane_slab_iterates(tmp_path, data_dir):
    """A few whole iterations of a slab through iterate_mc: at n_H = 1e4 the
    plane's Stromgren depth (~1e17 cm) lies inside the 3e18 cm slab, so the
    ionised layer forms at the lit face and the far side stays neutral."""
    from mocassin_xray_gb300 import iterate_mc
    s = Setup(configs.plane_slab(tmp_path / "dense", nh=1.0e4, nu_max=25.0), data_dir)
    ctx = Context(0)
    ctx.load(s)
    reps = iterate_mc(s, ctx, seed=3, n_photons=100000, max_iterations=3)
    assert len(reps) == 3
    i = s.info
    te = ctx.get(abi.ARR_TE)[1:].reshape(i.nx, i.ny, i.nz)
    assert np.all(np.isfinite(te)) and te[:, 0, :].mean() > 3000.0
    ion = ctx.get(abi.ARR_IONDEN).reshape(i.nstages, -1, s.n_cells + 1)
    xh1 = ion[1, 0, 1:].reshape(i.nx, i.ny, i.nz)       # X(H+)
    assert xh1[:, 0, :].mean() > xh1[:, -1, :].mean()
    ctx.close()


def test_xray_plane_slab_iterates(tmp_path, data_dir, oracle_lib):
    """The geometry of the reference's X-ray benchmarks: a plane-parallel slab
    lit by a hard power law to 740 Ryd, H to Fe with 31 stages (K shells and
    Auger yields): its FP64 transport equals the oracle's and whole
    production iterations run."""
    from mocassin_xray_gb300 import iterate_mc
    deck = configs.plane_slab(tmp_path / "xslab", nh=1.0e3, mean_field=2.9979e15, nu0=7.3529, nu0_add=0.56,
                              nu_max=740.0, abundances=configs.XRAY_ABUN, nstages=31,
                              cont_shape="powerlaw 1.5 1. 740.")
    s = Setup(deck, data_dir)
    assert s.info.plane_ionization == 1 and s.info.nstages == 31
    op = oracle_lib.opacity(s)
    rec = synthetic_recpdf(s.get(abi.ARR_NU), s.n_cells, seed=6)
    tl = np.full(s.n_cells + 1, 0.1, np.float32)
    ctx = Context(0)
    ctx.load(s)
    ctx.put(abi.ARR_OPACITY, op)
    ctx.put(abi.ARR_RECPDF, rec)
    ctx.put(abi.ARR_TOTAL_LINES, tl)
    n = 20000
    st = ctx.transport(n, seed=11, precision=abi.PREC_FP64)
    jo, _, so = oracle_lib.transport(s, op, rec, tl, n=n, seed=11, nthreads=8)
    assert st.crossings == so.crossings and st.escaped == so.escaped
    np.testing.assert_array_equal(ctx.get(abi.ARR_JSTE), jo)
    ctx.close()
    ctx = Context(0)
    ctx.load(s)
    reps = iterate_mc(s, ctx, seed=2, n_photons=50000, max_iterations=2)
    assert len(reps) == 2
    assert np.all(np.isfinite(ctx.get(abi.ARR_TE)[1:]))
    ctx.close()
