"""The query server (gg_server): mixed personalised-PageRank and BFS queries.

Every query is checked against the oracle (PPR within L1 <= 1e-6 of FP64,
BFS distances exact and parents forming a BFS tree), and every PPR result
must be bit-identical whether the query ran in a batch beside other queries
or alone.  A budget that holds two PPR results must bound the batches
without stalling the server.
"""
import numpy as np
import pytest

from graphs import pair

pytestmark = pytest.mark.gpu

DAMP = float(np.float32(0.85))
ITERS = 20


@pytest.fixture(scope="module")
def rg(gpu, orc):
    return pair(gpu, orc, gpu.Graph.rmat(12, 16))


def make_queries(V, deg, n, rng):
    nz = np.flatnonzero(deg)
    qs = []
    for _ in range(n):
        if rng.random() < 0.7:
            qs.append(("ppr", [int(x) for x in rng.integers(0, V, int(rng.integers(1, 33)))]))
        else:
            qs.append(("bfs", int(nz[rng.integers(0, len(nz))])))
    return qs


def submit(srv, q):
    kind, arg = q
    return srv.submit_ppr(arg) if kind == "ppr" else srv.submit_bfs(arg)


def test_server_mixed_queries_alone_and_together(gpu, orc, rg):
    g, o = rg
    dg = gpu.DeviceGraph(g, gpu.MAP_IN | gpu.MAP_OUT)
    srv = gpu.Server(dg, ppr_iterations=ITERS, ppr_storage="f32")
    qs = make_queries(g.V, g.arrays()["out_degree"], 60, np.random.default_rng(1))
    try:
        tickets = [submit(srv, q) for q in qs]
        mixed = [srv.take(t) for t in tickets]
        alone = [srv.take(submit(srv, q)) for q in qs]
    finally:
        srv.stop()
        dg.free()
    assert max(info["batch_size"] for (_, info), q in zip(mixed, qs) if q[0] == "ppr") > 1
    for i, (q, (rm, im), (ra, ia)) in enumerate(zip(qs, mixed, alone)):
        assert im["status"] == 0 and ia["status"] == 0
        assert im["submit_s"] <= im["start_s"] <= im["done_s"]
        kind, arg = q
        if kind == "ppr":
            assert ia["batch_size"] == 1
            np.testing.assert_array_equal(rm, ra, err_msg=f"query {i}")
            ex = orc.ppr_f64_multi(o, arg, ITERS, DAMP)
            assert np.abs(rm - ex).sum() <= 1e-6, i
        else:
            levels = orc.bfs_levels_reference(o, arg)
            for par, dist in (rm, ra):
                np.testing.assert_array_equal(dist, np.where(levels >= 0, levels, 0))
                orc.check_parents(o, arg, par, levels)
            assert im["bfs_reached"] == int((levels >= 0).sum())


def test_server_budget_bounds_batches(gpu, rg):
    g, _ = rg
    dg = gpu.DeviceGraph(g, gpu.MAP_IN | gpu.MAP_OUT)
    # room for one BFS result (8V) = two PPR results (4V each)
    srv = gpu.Server(dg, ppr_iterations=5, mem_budget_bytes=8 * g.V)
    try:
        tickets = [srv.submit_ppr([i]) for i in range(12)]
        infos = [srv.take(t, copy_out=False)[1] for t in tickets]
        t_bfs = srv.submit_bfs(0)
        _, ib = srv.take(t_bfs)
    finally:
        srv.stop()
        dg.free()
    assert all(i["status"] == 0 for i in infos) and ib["status"] == 0
    assert max(i["batch_size"] for i in infos) <= 2


def test_server_rejects_and_times_out(gpu, rg):
    g, _ = rg
    dg = gpu.DeviceGraph(g, gpu.MAP_IN | gpu.MAP_OUT)
    srv = gpu.Server(dg, ppr_iterations=5)
    try:
        with pytest.raises(gpu.GgError):
            srv.submit_bfs(g.V)
        with pytest.raises(gpu.GgError):
            srv.submit_ppr([g.V + 3])
        with pytest.raises(gpu.GgError):
            srv.take(123456)
    finally:
        srv.stop()
        dg.free()
    pull_only = gpu.DeviceGraph(g, gpu.MAP_IN)
    with pytest.raises(gpu.GgError):
        gpu.Server(pull_only, ppr_iterations=5)   # BFS needs the out-CSR too
    pull_only.free()


def test_server_ppr_equals_gg_ppr_alone(gpu, orc, rg):
    """A PPR query run in the server's continuous batch, beside others
    admitted and retired at other iterations, is bit-identical to gg_ppr on
    that seed set alone (FP32 and BF16 storage)."""
    g, o = rg
    rng = np.random.default_rng(21)
    sets = [[int(x) for x in rng.integers(0, g.V, int(rng.integers(1, 20)))] for _ in range(24)]
    for storage in ("f32", "bf16"):
        dg = gpu.DeviceGraph(g, gpu.MAP_IN | gpu.MAP_OUT)
        srv = gpu.Server(dg, ppr_iterations=ITERS, ppr_storage=storage)
        try:
            got = []
            tickets = []
            for i, s in enumerate(sets):
                tickets.append(srv.submit_ppr(s))
                if i % 5 == 4:   # take some while others run: slots retire and refill
                    got.append(srv.take(tickets.pop(0))[0])
            got += [srv.take(t)[0] for t in tickets]
        finally:
            srv.stop()
        for s, r in zip(sets, got):
            alone, _ = dg.ppr([s], iterations=ITERS, storage=storage)
            np.testing.assert_array_equal(r, alone[:, 0])
        dg.free()


def test_server_admits_between_iterations(gpu, orc):
    """Continuous batching: a query submitted while another is running
    starts before that one ends (at the next iteration boundary) instead of
    waiting for it, and both are exact."""
    import time

    g, o = pair(gpu, orc, gpu.Graph.rmat(16, 16))
    dg = gpu.DeviceGraph(g, gpu.MAP_IN | gpu.MAP_OUT)
    srv = gpu.Server(dg, ppr_iterations=400, ppr_storage="f32")
    try:
        t1 = srv.submit_ppr([1, 2])
        time.sleep(0.005)
        t2 = srv.submit_ppr([3])
        r1, i1 = srv.take(t1)
        r2, i2 = srv.take(t2)
    finally:
        srv.stop()
        dg.free()
    assert i2["start_s"] < i1["done_s"], (i1, i2)
    assert i2["batch_size"] == 2
    for r, s in ((r1, [1, 2]), (r2, [3])):
        assert np.abs(r - orc.ppr_f64_multi(o, s, 400, DAMP)).sum() <= 1e-5
