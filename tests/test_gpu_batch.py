"""PageRank over a batch of graphs (gg_pagerank_batch) and whole runs
launched as one CUDA graph (GG_PR_CUDA_GRAPH).

The batch is the block-diagonal union of small R-MAT graphs; each graph's
ranks must match the oracle's PageRank of that graph alone
(pageRank.c:942-1109, normalised by the graph's own vertex count).  A run
captured into a CUDA graph must give what the same run gives launch by
launch (bit for bit in the exact integer formats).
"""
import numpy as np
import pytest

from fpcheck import assert_fp_as_accurate
from graphs import pair

pytestmark = pytest.mark.gpu

SCALES = [5, 9, 7, 10, 6, 8]
SEED0 = 2024


@pytest.fixture(scope="module")
def batch(gpu):
    return gpu.Graph.rmat_batch(SCALES, edge_factor=8, seed0=SEED0)


@pytest.mark.parametrize("cuda_graph", [False, True])
def test_batch_pagerank_matches_each_graph(gpu, orc, batch, cuda_graph):
    g, voff = batch
    dg = gpu.DeviceGraph(g, gpu.MAP_IN)
    ranks, res = dg.pagerank_batch(voff, iterations=20, epsilon=0.0, cuda_graph=cuda_graph)
    dg.free()
    assert res["iterations"] == 20
    for i, sc in enumerate(SCALES):
        o = orc.rmat_csr(sc, 8, seed=SEED0 + i)
        ref, info = orc.pagerank(o, 0, 20, 0.0)
        ex = orc.pagerank_f64(o, info["executed"])
        assert_fp_as_accurate(ranks[voff[i]:voff[i + 1]], ref, ex, f"graph {i} (scale {sc})")


@pytest.mark.parametrize("mode", ["pull", "pull_fx64", "push", "dd_pull", "pull_q16"])
def test_cuda_graph_run_equals_launch_by_launch(gpu, orc, mode):
    g, o = pair(gpu, orc, gpu.Graph.rmat(12, 16))
    dg = gpu.DeviceGraph(g, gpu.MAP_ALL)
    a, ra = dg.pagerank(mode, iterations=20, epsilon=1e-4)
    b, rb = dg.pagerank(mode, iterations=20, epsilon=1e-4, cuda_graph=True)
    dg.free()
    assert ra["iterations"] == rb["iterations"]
    if mode in ("pull_fx64", "pull_q16"):
        np.testing.assert_array_equal(a, b)
    else:
        np.testing.assert_allclose(a, b, rtol=1e-5, atol=1e-12)


def test_batch_rejects_bad_arguments(gpu, batch):
    g, voff = batch
    dg = gpu.DeviceGraph(g, gpu.MAP_IN)
    with pytest.raises(gpu.GgError):
        dg.pagerank_batch(voff[:-1])            # does not reach V
    bad = voff.copy()
    bad[2] = bad[1]
    with pytest.raises(gpu.GgError):
        dg.pagerank_batch(bad)                  # an empty graph
    p = gpu.PrParams(0, 0, 20, 1, 0.0, 0.85, 0, 0)
    r = gpu.PrResult()
    assert gpu.lib().gg_pagerank_batch(dg.h, p, len(voff) - 1, voff.ctypes.data, None, r, None) == 1
    dg.free()


def test_cuda_graph_cache_reuse_and_invalidation(gpu):
    """GG_PR_CUDA_GRAPH keeps the instantiated graph on the mapping: a
    repeat call with the same parameters relaunches it and gives the same
    ranks; other parameters capture again; a BFS that regrows a shared work
    buffer in between forces a new capture (the old graph would write freed
    memory), and the ranks stay equal to the plain launches'."""
    g = gpu.Graph.rmat(14, 16)
    dg = gpu.DeviceGraph(g, gpu.MAP_IN | gpu.MAP_OUT)
    plain, _ = dg.pagerank("pull", iterations=20, epsilon=1e-4)
    a, ra = dg.pagerank("pull", iterations=20, epsilon=1e-4, cuda_graph=True)
    b, rb = dg.pagerank("pull", iterations=20, epsilon=1e-4, cuda_graph=True)
    np.testing.assert_allclose(a, plain, rtol=1e-6, atol=0)
    np.testing.assert_allclose(b, plain, rtol=1e-6, atol=0)
    assert ra["iterations"] == rb["iterations"] and ra["launches"] == rb["launches"]
    c, rc = dg.pagerank("pull", iterations=7, epsilon=0.0, cuda_graph=True)
    c_plain, rcp = dg.pagerank("pull", iterations=7, epsilon=0.0)
    np.testing.assert_allclose(c, c_plain, rtol=1e-6, atol=0)
    assert rc["iterations"] == rcp["iterations"] == 7
    dg.bfs(0, "do")  # regrows work buffer 0, which the captured graph also writes
    d, _ = dg.pagerank("pull", iterations=7, epsilon=0.0, cuda_graph=True)
    np.testing.assert_allclose(d, c_plain, rtol=1e-6, atol=0)
    e, _ = dg.pagerank("pull", iterations=20, epsilon=1e-4, storage="bf16", cuda_graph=True)
    e_plain, _ = dg.pagerank("pull", iterations=20, epsilon=1e-4, storage="bf16")
    np.testing.assert_allclose(e, e_plain, rtol=1e-6, atol=0)


@pytest.mark.parametrize("cfg", [(7, 16, 4096, 2), (7, 16, 0, 2), (5, 8, 200, 4), (9, 32, 512, 1), (7, 4, 64, 3)])
def test_many_graphs_kernel_per_graph_stop(gpu, orc, batch, cfg):
    """The many-graphs kernel (one CTA per graph, every iteration in one
    launch) with an epsilon stop: every graph stops on its own, after the
    iterations of the reference's loop on that graph alone, and its ranks
    pass the floating-point rule against the FP64 oracle.  The shapes cover
    every graph in shared memory, none, and a mix (bins at 64, 200 and 512
    vertices), with 5, 7 and 9 items per lane, 4 to 32 warps and 1 to 4
    resident CTAs per SM."""
    g, voff = batch
    dg = gpu.DeviceGraph(g, gpu.MAP_IN)
    dg.batch_config(*cfg, strategy=1)
    ranks, res = dg.pagerank_batch(voff, iterations=20, epsilon=1e-4)
    its = dg.batch_iterations(len(SCALES))
    dg.free()
    assert res["launches"] == 2 and res["gather_launches"] == 1
    for i, sc in enumerate(SCALES):
        o = orc.rmat_csr(sc, 8, seed=SEED0 + i)
        ref, info = orc.pagerank(o, 0, 20, 1e-4)
        assert its[i] == info["iterations"], (i, its[i], info["iterations"])
        ex = orc.pagerank_f64(o, info["executed"])
        assert_fp_as_accurate(ranks[voff[i]:voff[i + 1]], ref, ex, f"graph {i} (scale {sc}) cfg {cfg}")
    assert res["iterations"] == int(its.max())


def test_many_graphs_kernel_matches_union_run(gpu, batch):
    """With epsilon 0 every graph runs all iterations either way: the
    many-graphs kernel and the union pull agree to FP32 rounding."""
    g, voff = batch
    dg = gpu.DeviceGraph(g, gpu.MAP_IN)
    dg.batch_config(strategy=1)
    a, ra = dg.pagerank_batch(voff, iterations=20, epsilon=0.0)
    assert ra["gather_launches"] == 1
    b, rb = dg.pagerank_batch(voff, iterations=20, epsilon=0.0, union=True)
    dg.free()
    assert rb["gather_launches"] == 20
    np.testing.assert_allclose(a, b, rtol=2e-6, atol=0)


def test_many_graphs_kernel_rejects_edges_across_graphs(gpu, batch):
    """The kernel reads a small graph's contributions by local index, so a
    vertex_off that cuts a graph in two (edges cross the boundary) is
    refused, and the other shape configurations are checked on input."""
    g, voff = batch
    dg = gpu.DeviceGraph(g, gpu.MAP_IN)
    bad = voff.copy()
    bad[3] = (voff[3] + voff[4]) // 2   # splits graph 3
    with pytest.raises(gpu.GgError, match="cross"):
        dg.pagerank_batch(bad, iterations=5, epsilon=1e-4)  # an epsilon stop runs the kernel
    with pytest.raises(gpu.GgError):
        dg.batch_config(ipt=6)
    with pytest.raises(gpu.GgError):
        dg.batch_config(warps=32, smem_vmax=1 << 20)
    ok, _ = dg.pagerank_batch(voff, iterations=5, epsilon=1e-4)  # the right boundaries still work
    assert np.isfinite(ok).all()
    dg.free()
