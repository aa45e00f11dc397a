"""The multi-GPU bookkeeping of bench.py on CPU ranks (gloo, world size 2): every rank solves its own disjoint
batch of models (replicas, weak scaling), the timed region is the slowest rank's (MAX all-reduce) and the
whole-job value counts every rank's models over that time.  The GPU work itself is covered by the -m gpu
tests; nothing here touches a GPU."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    try:
        seeds = bench.rank_seeds(rank, 8)
        total = 2.0 + rank  # rank 1 is the slower one
        slowest = bench.max_over_ranks(total, world, device="cpu")
        gathered = [None] * world
        torch.distributed.all_gather_object(gathered, seeds)
        out[rank] = (seeds, slowest, bench.job_throughput(world, 8, 3, slowest), gathered)
    finally:
        torch.distributed.destroy_process_group()


def test_two_ranks_disjoint_batches_and_slowest_rank_time():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
    for r in range(world):
        seeds, slowest, value, gathered = out[r]
        assert seeds == list(range(8 * r, 8 * r + 8))
        assert slowest == 3.0  # the MAX over the ranks' times (2.0 and 3.0)
        assert value == pytest.approx(world * 8 * 3 / 3.0)
        assert not set(gathered[0]) & set(gathered[1])  # no model is solved twice
