"""Multi-process (N > 1) host logic of bench.py on CPU with gloo ranks.

The path has no exchange step (one domain per GPU; N ranks run N independent
replicas), so the only multi-rank logic is the timing protocol: a barrier on
both sides of the timed region and the maximum over ranks of the elapsed time.
"""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.barrier(dist)
        t = 1.5 + rank          # this rank's elapsed time
        out[rank] = bench.max_over_ranks(dist, t)
        bench.barrier(dist)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_max_over_ranks_with_gloo(world):
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_worker, args=(r, world, port, out)) for r in range(world)]
        for pr in procs:
            pr.start()
        for pr in procs:
            pr.join(timeout=120)
            assert pr.exitcode == 0
        assert dict(out) == {r: 1.5 + world - 1 for r in range(world)}


def test_chunk_count_matches_the_runtime_rule():
    import bench
    # display steps at 5, 100, 200, ..., 2500 -> 26 chunks
    assert bench.n_chunks(2500, 100) == 26
    assert bench.n_chunks(3, 100) == 1
    assert bench.n_chunks(300, 1000) == 1 + 3   # 5, then chunks of at most 128
