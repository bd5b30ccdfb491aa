"""The N > 1 host path of bench.py on CPU: two ranks over gloo (127.0.0.1).

bench.py runs one independent replica per GPU (the path shards by grids and sets, with
no data exchange); ranks meet only at the barriers around the timed region and in the
max over ranks of its duration, and only rank 0 runs the CPU reference arm.  These
tests run that logic with world size 2 and no GPU.
"""
import os
import socket

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import bench
    import torch.distributed as dist
    ws, r, local = bench._dist()
    bench._barrier(ws)
    t = bench._max_over_ranks(ws, 1.5 + r)  # each rank's "duration"
    # the reference arm: rank 0 alone runs and prints; the others return at once
    class Args:
        steps, warmup = 1, 0
    other = bench.run_reference(Args, ws, r) if r != 0 else None
    bench._barrier(ws)
    dist.destroy_process_group()
    q.put((r, ws, local, t, other))


def test_two_rank_barrier_and_max_over_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    assert all(o[1] == 2 for o in out)
    assert [o[2] for o in out] == [0, 1]
    # every rank reports the slowest rank's time
    assert all(o[3] == pytest.approx(2.5) for o in out)
    # rank 1 does not run the reference arm
    assert out[1][4] == 0
