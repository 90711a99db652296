"""The N > 1 path of bench.py (replicas, one process per GPU) exercised with
two gloo ranks on the CPU: the barrier, the max of the ranks' times and the
whole-job value the bench reports (every rank's units over the slowest rank's
time).  No GPU and no collective on a data path are involved."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench

    reps = bench.Replicas(world, "gloo", "cpu")
    reps.barrier()
    local_ms = 100.0 * (rank + 1)          # rank 1 is the slowest
    slowest = reps.max(local_ms)
    value = reps.value(1e9, slowest)
    reps.barrier()
    reps.close()
    out.put((rank, slowest, value, bench.dist_env()))


def test_replicas_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, slowest, value, env in res:
        assert slowest == 200.0                         # max over ranks
        assert abs(value - 2 * 1e9 / 0.2) < 1e-3 * value  # both ranks' units over the slowest time
        assert env == (2, rank, rank)


def test_replicas_single_process_needs_no_process_group():
    import bench

    reps = bench.Replicas(1)
    reps.barrier()
    assert reps.max(3.5) == 3.5
    assert reps.value(10.0, 1000.0) == 10.0
    reps.close()
