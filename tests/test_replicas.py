"""CPU test of the multi-GPU path of bench.py (replicas only: one independent
solve per GPU, no data-path collective): two gloo ranks on 127.0.0.1 exercise
the barrier and the max/sum reductions that turn per-rank timings into the
whole-job number, and the reference arm runs on rank 0 only."""
import multiprocessing as mp
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    import bench
    d = bench.Dist(ws)
    d.barrier()
    # rank r: (1 + r) seconds for 1e6 * (r + 1) DOF x iterations
    value, tmax = bench.replica_throughput(d, 1.0 + rank, 1e6 * (rank + 1))
    skipped = bench.run_reference_arm(None, None, ws, rank) if rank else "rank0"
    d.barrier()
    d.close()
    q.put((rank, value, tmax, skipped))


def test_two_replicas_reduce_like_the_bench():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, tmax, skipped in out:
        assert tmax == 2.0                      # the slowest rank's time
        assert value == pytest.approx(3e6 / 2.0 / 1e6)  # all ranks' work over it
    assert out[1][3] is None                    # the reference arm does no work off rank 0
