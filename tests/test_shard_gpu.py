"""A sharded MC iteration through libmcx: two ranks (gloo on the host; both
on the one GPU of the machine, their kernels independent of each other) each
transport their counter range of an iteration's packets, sum Jste and the
escape tallies (shard.transport_sharded, the reference's MPI_Allreduce of
source/iteration_mod.f90:953) and balance every cell.  The summed estimators
and the event counts equal a single-rank run of all the packets, and so does
the balance that follows."""
import os
import socket

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, deck, data_dir, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from mocassin_xray_gb300 import Context, Setup, abi, iterate_mc
    s = Setup(deck, data_dir)
    ctx = Context(0)
    ctx.load(s)
    rep = iterate_mc(s, ctx, seed=21, n_photons=20000, max_iterations=1, precision=abi.PREC_FP64, group=True)
    if rank == 0:
        np.save(os.path.join(out_dir, "j.npy"), ctx.get(abi.ARR_JSTE))
        np.save(os.path.join(out_dir, "te.npy"), ctx.get(abi.ARR_TE))
        np.save(os.path.join(out_dir, "counts.npy"), np.array([rep[0].transport[k] for k in sorted(rep[0].transport)]))
    ctx.close()
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_iterate_like_one(decks, data_dir, tmp_path):
    import torch.multiprocessing as mp
    from mocassin_xray_gb300 import Context, Setup, abi, iterate_mc
    deck = decks["lognormal_small"]
    mp.start_processes(_rank_main, args=(2, _free_port(), str(deck), str(data_dir), str(tmp_path)), nprocs=2,
                       join=True, start_method="spawn")
    s = Setup(deck, data_dir)
    ctx = Context(0)
    ctx.load(s)
    rep = iterate_mc(s, ctx, seed=21, n_photons=20000, max_iterations=1, precision=abi.PREC_FP64)
    counts = np.array([rep[0].transport[k] for k in sorted(rep[0].transport)])
    np.testing.assert_array_equal(np.load(tmp_path / "counts.npy"), counts)
    # each rank's J is its own correctly rounded sum: the two add with one more rounding
    np.testing.assert_allclose(np.load(tmp_path / "j.npy"), ctx.get(abi.ARR_JSTE), rtol=1e-15, atol=0)
    np.testing.assert_allclose(np.load(tmp_path / "te.npy"), ctx.get(abi.ARR_TE), rtol=1e-6)
    ctx.close()
