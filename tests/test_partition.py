"""Replica sharding of independent right-hand sides (parallel.f90:80-135),
exercised with world_size 2 gloo ranks on the CPU like parallel.pf's npes tests."""
import os

import pytest

from sternheimergw_gb300.parallel import parallel_task


@pytest.mark.parametrize("size", [1, 2, 3, 4])
def test_parallel_task_blocks(size):
    for total in (0, 1, 5, 113, 1808):
        got = [parallel_task(total, r, size) for r in range(size)]
        counts = got[0][2]
        assert sum(counts) == total and len(counts) == size
        assert counts == sorted(counts)  # the last ranks carry the remainder
        first = 0
        for r, (a, b, _) in enumerate(got):
            assert a == first and b - a + 1 == counts[r]
            first = b + 1


def _worker(rank, size, port, out):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=size)
    first, last, counts = parallel_task(113, rank, size)
    # each rank "solves" its block; the host-side gather pads to equal sizes (gloo all_gather)
    mine = torch.arange(first, last + 1, dtype=torch.int64)
    width = max(counts)
    padded = torch.full((width,), -1, dtype=torch.int64)
    padded[:mine.numel()] = mine
    gathered = [torch.zeros(width, dtype=torch.int64) for _ in counts]
    dist.all_gather(gathered, padded)
    if rank == 0:
        out.put(torch.cat([g[:c] for g, c in zip(gathered, counts)]).tolist())
    dist.barrier()
    dist.destroy_process_group()


def test_gloo_two_ranks_cover_all_tasks():
    import socket

    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    result = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert result == list(range(113))
