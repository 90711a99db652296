"""Size-independent properties at the measured workloads' full sizes, where
the oracle would take minutes per case:

* R-MAT-22 undirected (the BFS workload, V 4.2M, E 134M): every search
  reaches exactly its source's connected component (connected components
  and BFS computed independently), and levels differ by at most one across
  every edge;
* R-MAT-24 (the PageRank workload, V 16.8M, E 268M): the CSR built on the
  device is identical to the host build, and FP32 PageRank agrees with the
  fixed-point (Q32.32, exact integer sums) variant to FP32 rounding."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEED = 27491095


def test_bfs_reaches_exactly_the_component_rmat22u(gpu):
    g = gpu.Graph.rmat(22, 16, seed=SEED, symmetric=True)
    dg = gpu.DeviceGraph(g, gpu.MAP_IN | gpu.MAP_OUT)
    comp, cres = dg.cc("afforest", use_in_edges=0)
    v = g.views()
    src = v["out_adj"]
    row = np.repeat(np.arange(g.V, dtype=np.uint32), v["out_degree"].astype(np.int64))
    rng = np.random.default_rng(5)
    deg = v["out_degree"]
    for s in rng.choice(np.flatnonzero(deg), 4, replace=False):
        s = int(s)
        parents, dist, r = dg.bfs(s, "do")
        reached = parents >= 0
        np.testing.assert_array_equal(reached, comp == comp[s])
        assert r["processed_nodes"] == int(reached.sum())  # the source is counted, as in the reference
        # BFS levels: along every edge between reached vertices they differ by <= 1
        both = reached[row] & reached[src]
        gap = np.abs(dist[row[both]].astype(np.int64) - dist[src[both]].astype(np.int64))
        assert int(gap.max()) <= 1
    dg.free()
    g.free()


def test_device_build_and_fixed_point_agreement_rmat24(gpu):
    g_host = gpu.Graph.rmat(24, 16, seed=SEED)
    g_dev = gpu.Graph.rmat(24, 16, seed=SEED, device_build=True)
    a, b = g_host.arrays(), g_dev.arrays()
    for k in ("out_off", "out_adj", "in_off", "in_adj", "out_degree", "in_degree"):
        assert np.array_equal(a[k], b[k]), k
    g_dev.free()
    dg = gpu.DeviceGraph(g_host, gpu.MAP_IN)
    f32, r1 = dg.pagerank("pull", iterations=20, epsilon=0.0)
    fx, r2 = dg.pagerank("pull_fx64", iterations=20, epsilon=0.0)
    assert r1["iterations"] == r2["iterations"] == 20
    l1 = float(np.abs(f32.astype(np.float64) - fx).sum()) / float(np.abs(fx).sum())
    assert l1 <= 1e-5, l1
    dg.free()
    g_host.free()
