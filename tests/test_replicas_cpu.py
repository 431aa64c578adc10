"""The multi-rank bench path (replicas only) on CPU: two gloo ranks agree on the max-over-ranks
time, each rank gets its own seed, and no data-path collective is involved."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    import bench

    w, r, local = bench.dist_setup()
    bench.barrier(w)
    t = bench.all_max(w, 1.0 + rank)
    out[rank] = (w, r, local, t, 20261203 + r)
    import torch.distributed as dist

    dist.destroy_process_group()


def test_two_gloo_ranks_max_over_ranks():
    world, port = 2, _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
    assert sorted(out.keys()) == [0, 1]
    for rank in range(world):
        w, r, local, t, seed = out[rank]
        assert (w, r, local) == (world, rank, rank)
        assert t == 2.0  # the slowest rank's time
    assert out[0][4] != out[1][4]  # independent replicas
