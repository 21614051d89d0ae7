"""Batches of nebulae (mcx_load_batched / mcx_transport_batched / mcx_iterate_batched): every nebula of
a batch gives what a context holding that nebula alone gives."""
import numpy as np
import pytest

from mocassin_xray_gb300 import abi, configs, Context, Setup

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch_setups(tmp_path_factory, data_dir):
    root = tmp_path_factory.mktemp("batch")
    decks = configs.nebula_batch(root, n=4, seed=5, packets_range=(1e4, 4e4), octant_every=2, max_edge=17)
    return [Setup(d, data_dir, mesh_mode=abi.MESH_LOG_EDGES) for d, _ in decks], [pk for _, pk in decks]


def test_batch_phases_equal_single_nebula_runs(batch_setups):
    setups, packets = batch_setups
    seeds = [101 + b for b in range(len(setups))]
    bc = Context(0)
    bc.load_batched(setups)
    assert list(bc.cell_offsets) == list(np.cumsum([0] + [s.info.n_cells for s in setups]))
    bc.opacity(1)
    bc.emission(1)
    bst = bc.transport_batched(packets, seeds, precision=abi.PREC_FP64)
    bc.normalize_j()
    jb, ob, rb = bc.get(abi.ARR_JSTE), bc.get(abi.ARR_OPACITY), bc.get(abi.ARR_RECPDF)
    bc.balance()
    teb = bc.get(abi.ARR_TE)
    esc_total = 0
    for b, s in enumerate(setups):
        sc = Context(0)
        sc.load(s)
        sc.opacity(1)
        sc.emission(1)
        st = sc.transport(packets[b], seed=seeds[b], precision=abi.PREC_FP64)
        esc_total += st.escaped
        sc.normalize_j()
        # per-cell phases: the same bits (each nebula keeps its own Gaunt cache)
        np.testing.assert_array_equal(bc.nebula_cells(ob, b), sc.get(abi.ARR_OPACITY)[:, 1:])
        np.testing.assert_array_equal(bc.nebula_cells(rb, b), sc.get(abi.ARR_RECPDF)[:, 1:])
        # transport: the same histories; FP64 atomics add them in another order
        np.testing.assert_allclose(bc.nebula_cells(jb, b), sc.get(abi.ARR_JSTE)[:, 1:], rtol=1e-10, atol=0)
        sc.balance()
        ts = sc.get(abi.ARR_TE)[1:]
        same = np.abs(bc.nebula_cells(teb, b) - ts) <= 1e-6 * ts
        assert same.mean() >= 0.99
        sc.close()
    assert bst.escaped == esc_total
    bc.close()


def test_iterate_batched_runs_every_nebula(batch_setups):
    setups, packets = batch_setups
    bc = Context(0)
    bc.load_batched(setups)
    for it in (1, 2):
        st = bc.iterate_batched(packets, [7] * len(setups), [(it - 1) << 40] * len(setups), n_iterate_mc=it)
        assert st.transport.emissions >= sum(packets)
        assert st.balance.cells_updated + st.balance.no_hit == bc.cell_offsets[-1]
    te = bc.get(abi.ARR_TE)
    for b in range(len(setups)):
        assert np.all(np.isfinite(bc.nebula_cells(te, b)))
    with pytest.raises(RuntimeError, match="batch"):
        bc.transport(1000)
    bc.close()


def test_incompatible_nebulae_are_rejected(batch_setups, decks, data_dir):
    setups, _ = batch_setups
    other = Setup(decks["h_small"], data_dir)          # 400-bin mesh
    bc = Context(0)
    with pytest.raises(RuntimeError, match="frequency mesh"):
        bc.load_batched([setups[0], other])
    bc.close()


def test_line_luminosities_per_nebula(batch_setups):
    """mcx_line_luminosities_nebula sums one nebula's cells in the same groups as a context holding that
    nebula alone: the same bits."""
    setups, _ = batch_setups
    bc = Context(0)
    bc.load_batched(setups)
    for b, s in enumerate(setups):
        sc = Context(0)
        sc.load(s)
        g1 = bc.line_luminosities(nebula=b)
        g2 = sc.line_luminosities()
        assert g1["n_cells"] == g2["n_cells"] == s.info.n_cells
        assert g1["hbeta_vol"] == g2["hbeta_vol"]
        for key in ("hydro", "hei", "te_vol", "ion_vol"):
            np.testing.assert_array_equal(g1[key], g2[key])
        sc.close()
    with pytest.raises(RuntimeError, match="batch"):
        bc.line_luminosities()
    bc.close()


def test_batch_timers_and_tuned_launch(data_dir, tmp_path):
    """Each nebula's finishing time within the batched launch lies inside the
    launch, and the autotuned launch shape gives the same J bits as the default
    one (the shape changes the schedule, never a history)."""
    from mocassin_xray_gb300 import autotune
    decks = configs.nebula_batch(tmp_path, n=6, seed=3, max_edge=13, packets_range=(5e3, 2e4))
    setups = [Setup(d, data_dir, mesh_mode=abi.MESH_LOG_EDGES) for d, _ in decks]
    packets = np.array([pk for _, pk in decks], dtype=np.int64)
    seeds = np.arange(len(decks), dtype=np.uint64) + np.uint64(40)
    ctx = Context(0)
    ctx.load_batched(setups)
    ctx.opacity(1)
    ctx.emission(1)
    st = ctx.transport_batched(packets, seeds)
    j0 = ctx.get(abi.ARR_JSTE)
    ms = ctx.batch_transport_ms()
    assert ms.shape == (len(setups),)
    assert np.all(ms > 0) and ms.max() <= st.kernel_ms * 1.05 + 0.05

    def run(L):
        return ctx.transport_batched(packets, seeds, block_size=L["block_size"], grid_mult=L["grid_mult"],
                                     emit_batch=L["emit_batch"]).kernel_ms

    tuned = autotune.tune_transport(run, reps=1)
    ctx.transport_batched(packets, seeds, **autotune.launch_of(tuned))
    np.testing.assert_array_equal(ctx.get(abi.ARR_JSTE), j0)
    ctx.close()
