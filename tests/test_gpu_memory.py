"""Memory reuse between calls: the device-block cache and the recycled host
arrays of the stats structs.

* A mapping made and dropped repeatedly (what every drop-in call on a host
  graph does) takes its blocks from the cache after the first round: device
  memory in use stays flat, the cache holds the blocks between rounds, and
  the results stay bit-identical (fixed-point PageRank, integer sums).
* gg_device_cache_trim empties the cache and gives the memory back.
* Stats arrays are recycled between drop-in calls, and a recycled array
  handed to newPageRankStatsGraphCSR is initialised as the reference
  initialises a fresh one (base_pr ranks, realRanks[v] = v).
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _free_bytes():
    import torch

    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def test_map_unmap_reuses_cached_blocks(gpu):
    g = gpu.Graph.rmat(18, 16)
    gpu.device_cache_trim()
    first, free_after = None, []
    for _ in range(5):
        dg = gpu.DeviceGraph(g, gpu.MAP_IN)
        ranks, _ = dg.pagerank("pull_fx64", iterations=10)
        held = dg.device_bytes()
        dg.free()
        assert gpu.device_cache_bytes() >= held > 0
        free_after.append(_free_bytes())
        if first is None:
            first = ranks
        else:
            np.testing.assert_array_equal(ranks, first)
    # after the first round every block comes from the cache
    assert len(set(free_after[1:])) == 1, free_after
    before = _free_bytes()
    gpu.device_cache_trim()
    assert gpu.device_cache_bytes() == 0
    assert _free_bytes() > before


def test_cached_blocks_serve_a_different_graph(gpu, orc):
    """Blocks cached from one graph's mapping serve another graph's of a
    different size; the results are the oracle's."""
    from graphs import pair

    big = gpu.Graph.rmat(17, 16)
    gpu.DeviceGraph(big, gpu.MAP_ALL).free()
    g, o = pair(gpu, orc, gpu.Graph.rmat(16, 8))
    dg = gpu.DeviceGraph(g, gpu.MAP_IN | gpu.MAP_OUT)
    _, dist, _ = dg.bfs(3, "do")
    _, rd, _ = orc.bfs(o, 2, 3)
    np.testing.assert_array_equal(dist, rd)
    ranks, info = dg.pagerank("pull_fx64", iterations=20, epsilon=1e-4)
    dg.free()
    ref, rinfo = orc.pagerank(o, 2, 20, 1e-4)
    assert info["iterations"] == rinfo["iterations"]
    np.testing.assert_array_equal(ranks, ref)


def test_stats_arrays_recycled_and_initialised(gpu):
    L = gpu.lib()
    g = gpu.Graph.rmat(18, 16)   # V = 262144: 1 MiB arrays (recycled from 64 KiB)
    args = gpu.default_arguments(iterations=5, epsilon=0.0)
    gpu.set_gpu_options(storage="f32", device=0, keep_resident=False, verbose=False)
    s1 = L.pageRankGraphCSR(C.byref(args), g.ptr)
    assert s1
    p1 = C.cast(s1.contents.pageRanks, C.c_void_p).value
    ranks1 = np.ctypeslib.as_array(s1.contents.pageRanks, (g.V,)).copy()
    L.freePageRankStats(s1)
    s2 = L.pageRankGraphCSR(C.byref(args), g.ptr)
    assert s2
    ranks2 = np.ctypeslib.as_array(s2.contents.pageRanks, (g.V,)).copy()
    rr = np.ctypeslib.as_array(s2.contents.realRanks, (g.V,)).copy()
    recycled = {C.cast(s2.contents.pageRanks, C.c_void_p).value, C.cast(s2.contents.realRanks, C.c_void_p).value}
    L.freePageRankStats(s2)
    assert p1 in recycled
    np.testing.assert_array_equal(rr, np.arange(g.V, dtype=np.uint32))
    # FP32 pull sums spanning rows in arrival order: equal within rounding
    np.testing.assert_allclose(ranks2, ranks1, rtol=1e-5, atol=1e-12)
    # a recycled array (holding the last call's ranks) given to the public
    # constructor comes back initialised
    s3 = L.newPageRankStatsGraphCSR(g.ptr)
    st = s3.contents
    pr = np.ctypeslib.as_array(st.pageRanks, (g.V,))
    assert (pr == np.float32(st.base_pr)).all()
    np.testing.assert_array_equal(np.ctypeslib.as_array(st.realRanks, (g.V,)), np.arange(g.V, dtype=np.uint32))
    L.freePageRankStats(s3)
