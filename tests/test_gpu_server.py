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
