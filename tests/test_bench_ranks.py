"""bench.py's multi-GPU path is replicas (one simulation batch per rank, no
collective on the data path) timed by the slowest rank: the rank set-up and
the max-over-ranks reduction, run here as two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import bench

    class Args:
        impl = "reference"   # the gloo arm of dist_setup

    w, r, local = bench.dist_setup(Args)
    assert (w, r, local) == (world, rank, rank)
    got = bench.max_over_ranks(10.0 * (rank + 1), w)
    out.put((rank, got))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(out.get(timeout=10) for _ in range(2))
    assert got == [(0, 20.0), (1, 20.0)]


def test_single_rank_is_identity():
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
