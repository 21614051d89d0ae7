"""Packets shard by counter range across ranks with one sum of J (world size 2, gloo, on the host):
the reduced estimators equal a single-rank run of all the packets."""
import os
import socket

import numpy as np
import pytest

from mocassin_xray_gb300.shard import shard_packets


def test_shard_ranges_partition_the_packets():
    for n in (0, 1, 7, 1000, 10_000_001):
        for world in (1, 2, 3, 8):
            ranges = [shard_packets(n, r, world) for r in range(world)]
            assert sum(c for _, c in ranges) == n
            assert ranges[0][0] == 0
            for (f0, c0), (f1, _) in zip(ranges, ranges[1:]):
                assert f0 + c0 == f1
            assert max(c for _, c in ranges) - min(c for _, c in ranges) <= 1
    with pytest.raises(ValueError):
        shard_packets(10, 2, 2)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, deck, data_dir, n, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import oracle
    from mocassin_xray_gb300 import Setup
    from mocassin_xray_gb300.shard import allreduce_sum, shard_packets
    s = Setup(deck, data_dir)
    op = oracle.opacity(s)
    rec = np.load(os.path.join(out_dir, "rec.npy"))
    tl = np.load(os.path.join(out_dir, "tl.npy"))
    first, count = shard_packets(n, rank, world)
    j, esc, _ = oracle.transport(s, op, rec, tl, n=count, seed=9, counter_base=first, n_photons_norm=n)
    j = allreduce_sum(j)
    esc = allreduce_sum(esc)
    if rank == 0:
        np.save(os.path.join(out_dir, "j_sharded.npy"), j)
        np.save(os.path.join(out_dir, "esc_sharded.npy"), esc)
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_sum_to_the_single_run(decks, data_dir, oracle_lib, tmp_path):
    import torch.multiprocessing as mp
    from conftest import synthetic_recpdf
    from mocassin_xray_gb300 import abi, Setup
    s = Setup(decks["h_small"], data_dir)
    n = 6000
    rec = synthetic_recpdf(s.get(abi.ARR_NU), s.info.n_cells, seed=2)
    tl = np.zeros(s.info.n_cells + 1, np.float32)
    np.save(tmp_path / "rec.npy", rec)
    np.save(tmp_path / "tl.npy", tl)
    op = oracle_lib.opacity(s)
    j1, esc1, _ = oracle_lib.transport(s, op, rec, tl, n=n, seed=9, counter_base=0)
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, str(decks["h_small"]), str(data_dir), n, str(tmp_path)))
             for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    j2 = np.load(tmp_path / "j_sharded.npy")
    esc2 = np.load(tmp_path / "esc_sharded.npy")
    np.testing.assert_allclose(j2, j1, rtol=1e-12, atol=0)
    np.testing.assert_allclose(esc2, esc1, rtol=1e-12, atol=0)
    assert j1.sum() > 0
