"""The pull gather through the hot-vertex table (GG_PR_HOT_ON): the 16K
vertices with the most out-edges are read from shared memory through a
flag-encoded copy of the CSC ids.  The table holds exact copies, so the
ranks obey the same FP rule against the oracle as the plain gather, and
agree with the plain gather up to the order in which rows spanning tiles add
their partials.  Graphs smaller than the table (every vertex hot) and a hub
graph whose hot rows span many tiles are covered."""
import numpy as np
import pytest

from fpcheck import assert_fp_as_accurate
from graphs import pair, special_edges

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def graphs(gpu, orc):
    src, dst, w, V = special_edges()["hubs"]
    return {"rmat12": pair(gpu, orc, gpu.Graph.rmat(12, 16)),
            "rmat16": pair(gpu, orc, gpu.Graph.rmat(16, 16)),
            "hubs": pair(gpu, orc, gpu.Graph.from_edges(src, dst, w, num_vertices=V))}


@pytest.mark.parametrize("name", ["rmat12", "rmat16", "hubs"])
@pytest.mark.parametrize("storage", ["f32", "bf16", "f16"])
def test_hot_table_pull(gpu, orc, graphs, name, storage):
    g, o = graphs[name]
    dg = gpu.DeviceGraph(g, gpu.MAP_IN)
    hot, rh = dg.pagerank("pull", storage=storage, iterations=20, epsilon=1e-4, hot=True)
    plain, rp = dg.pagerank("pull", storage=storage, iterations=20, epsilon=1e-4, hot=False)
    dg.free()
    assert rh["iterations"] == rp["iterations"]
    np.testing.assert_allclose(hot, plain, rtol=2e-6, atol=1e-12)
    if storage == "f32":
        ref, info = orc.pagerank(o, 0, 20, 1e-4)
        assert rh["iterations"] == info["iterations"]
        assert_fp_as_accurate(hot, ref, orc.pagerank_f64(o, info["executed"]), f"{name} hot")


def test_hot_table_in_a_cuda_graph_run(gpu, orc, graphs):
    g, o = graphs["rmat16"]
    dg = gpu.DeviceGraph(g, gpu.MAP_IN)
    a, _ = dg.pagerank("pull", iterations=20, epsilon=0.0, hot=True, cuda_graph=True)
    b, _ = dg.pagerank("pull", iterations=20, epsilon=0.0, hot=True)
    dg.free()
    np.testing.assert_allclose(a, b, rtol=2e-6, atol=1e-12)


@pytest.mark.parametrize("name", ["rmat12", "hubs"])
@pytest.mark.parametrize("storage", ["f32", "bf16", "f16"])
def test_hot_table_spmv_pull(gpu, orc, graphs, name, storage):
    g, o = graphs[name]
    if name == "rmat12":
        g, o = pair(gpu, orc, gpu.Graph.rmat(12, 16, weighted=True))
    dg = gpu.DeviceGraph(g, gpu.MAP_IN | gpu.MAP_IN_W)
    x = np.random.default_rng(9).random(g.V).astype(np.float32)
    _, hot, _ = dg.spmv("pull", storage=storage, x=x, hot=True)
    _, plain, _ = dg.spmv("pull", storage=storage, x=x, hot=False)
    dg.free()
    np.testing.assert_allclose(hot, plain, rtol=2e-6, atol=1e-9)
    if storage == "f32":
        _, y32, _ = orc.spmv(o, 0, 1, x=x)
        assert_fp_as_accurate(hot, y32, orc.spmv_f64(o, x), f"{name} spmv hot")
