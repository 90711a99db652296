"""The reference-compatible C entry points (pageRank*GraphCSR,
breadthFirstSearch*GraphCSR, SPMV*GraphCSR and the BFS step functions)
called through the C ABI, checked against the oracle -- the way the
reference's own test driver compares variants (test_open-graph-match.c:94-146)."""
import ctypes as C

import numpy as np
import pytest

from fpcheck import assert_fp_as_accurate
from graphs import pair

pytestmark = pytest.mark.gpu

PR_FNS = ["pageRankPullGraphCSR", "pageRankPushGraphCSR", "pageRankPullFixedPoint64BitGraphCSR",
          "pageRankPushFixedPointGraphCSR", "pageRankPullQuant32BitGraphCSR", "pageRankPushQuantGraphCSR",
          "pageRankDataDrivenPullGraphCSR", "pageRankDataDrivenPushGraphCSR",
          "pageRankDataDrivenPullPushGraphCSR", "pageRankPullFixedPoint32BitGraphCSR",
          "pageRankPullFixedPoint16BitGraphCSR", "pageRankPullFixedPoint8BitGraphCSR",
          "pageRankPullQuant16BitGraphCSR", "pageRankPullQuant8BitGraphCSR"]
BFS_FNS = ["breadthFirstSearchPullGraphCSR", "breadthFirstSearchPushGraphCSR",
           "breadthFirstSearchDirectionOptimizedGraphCSR", "breadthFirstSearchPushBitmapGraphCSR",
           "breadthFirstSearchPushDirectionOptimizedBitmapGraphCSR"]
SPMV_FNS = ["SPMVPullGraphCSR", "SPMVPushGraphCSR", "SPMVPullFixedPointGraphCSR", "SPMVPushFixedPointGraphCSR"]


@pytest.fixture(scope="module")
def rg(gpu, orc):
    gpu.set_gpu_options()
    return pair(gpu, orc, gpu.Graph.rmat(12, 16, weighted=True))


@pytest.mark.parametrize("mode", list(range(14)))
def test_pagerank_dispatch_and_named(gpu, orc, rg, mode):
    g, o = rg
    a = gpu.default_arguments(iterations=20, epsilon=1e-4, pushpull=mode)
    r1, s1 = gpu.pagerank_csr(g, a, "pageRankGraphCSR")
    r2, s2 = gpu.pagerank_csr(g, gpu.default_arguments(iterations=20, epsilon=1e-4), PR_FNS[mode])
    ref, info = orc.pagerank(o, mode, 20, 1e-4)
    assert s1["damp"] == np.float32(0.85) and s1["base_pr"] == np.float32(1.0) - np.float32(0.85)
    np.testing.assert_array_equal(s1["realRanks"], np.arange(g.V, dtype=np.uint32))
    if mode in (7, 8):
        return
    assert s1["iterations"] == info["iterations"] == s2["iterations"]
    if mode in (2, 3, 4, 9, 10, 11, 12, 13):
        np.testing.assert_array_equal(r1, ref)
        np.testing.assert_array_equal(r2, ref)
    elif mode in (0, 1):
        ex = orc.pagerank_f64(o, info["executed"])
        assert_fp_as_accurate(r1, ref, ex, f"mode {mode}")
        assert_fp_as_accurate(r2, ref, ex, f"mode {mode}")
    elif mode == 6:
        assert float(np.abs(r1 - ref).max()) <= 2e-4 * float(ref.max())
    else:
        assert float(np.abs(r1 - ref).sum()) <= 5e-3 * float(np.abs(ref).sum())


def test_pagerank_unknown_code_falls_back_to_pull(gpu, orc, rg):
    g, o = rg
    r, s = gpu.pagerank_csr(g, gpu.default_arguments(pushpull=99))
    ref, info = orc.pagerank(o, 0, 20, 1e-4)
    assert s["iterations"] == info["iterations"]


@pytest.mark.parametrize("mode", list(range(5)))
def test_bfs_dispatch_and_named(gpu, orc, rg, mode):
    g, o = rg
    for src in (0, 5, g.V - 1):
        a = gpu.default_arguments(source=src, pushpull=mode)
        p1, d1, s1 = gpu.bfs_csr(g, a)
        p2, d2, s2 = gpu.bfs_csr(g, gpu.default_arguments(source=src), BFS_FNS[mode])
        rp, rd, info = orc.bfs(o, mode, src)
        np.testing.assert_array_equal(d1, rd)
        np.testing.assert_array_equal(d2, rd)
        assert s1["processed_nodes"] == info["processed_nodes"] == s2["processed_nodes"]
        assert s1["iteration"] == info["iteration"]
        assert s1["source"] == src  # label_array is the identity


def test_bfs_out_of_range_source_returns_initial_stats(gpu, rg):
    g, o = rg
    a = gpu.default_arguments(source=g.V + 5)
    p, d, s = gpu.bfs_csr(g, a)
    deg = np.diff(o.out_off.astype(np.int64))
    np.testing.assert_array_equal(p, np.where(deg > 0, -deg, -1).astype(np.int32))
    assert not d.any() and s["processed_nodes"] == 0
    a = gpu.default_arguments(source=-3)  # negative compares as a huge unsigned
    p, d, s = gpu.bfs_csr(g, a)
    assert s["processed_nodes"] == 0


@pytest.mark.parametrize("mode", list(range(4)))
def test_spmv_dispatch_and_named(gpu, orc, rg, mode):
    g, o = rg
    x1, y1, s1 = gpu.spmv_csr(g, gpu.default_arguments(iterations=4, pushpull=mode))
    x2, y2, s2 = gpu.spmv_csr(g, gpu.default_arguments(iterations=4), SPMV_FNS[mode])
    rx, ry, _ = orc.spmv(o, mode, 4)
    np.testing.assert_array_equal(x1, rx)
    assert s1["iterations"] == 4
    if mode in (2, 3):
        np.testing.assert_array_equal(y1, ry)
        np.testing.assert_array_equal(y2, ry)
    else:
        ex = orc.spmv_f64(o, rx) * (4 if mode == 1 else 1)
        assert_fp_as_accurate(y1, ry, ex, f"mode {mode}")


def test_resident_mapping_and_release(gpu, orc, rg):
    g, o = rg
    gpu.set_gpu_options(keep_resident=True)
    try:
        r1, _ = gpu.pagerank_csr(g, gpu.default_arguments())
        r2, _ = gpu.pagerank_csr(g, gpu.default_arguments())
        assert float(np.abs(r1 - r2).max()) <= 1e-5 * float(r1.max())
        gpu.lib().graphGpuRelease(g.ptr)
    finally:
        gpu.set_gpu_options()


def test_step_functions_drive_a_bfs(gpu, orc, rg):
    """A caller-driven BFS over topDownStepGraphCSR / bottomUpStepGraphCSR,
    the loop of breadthFirstSearchDirectionOptimizedGraphCSR (BFS.c:592-646)."""
    g, o = rg
    L = gpu.lib()
    src = 0
    stats = L.newBFSStatsGraphCSR(g.ptr)
    q = L.newArrayQueue(g.V)
    cur, nxt = L.newBitmap(g.V), L.newBitmap(g.V)
    try:
        stats.contents.parents[src] = src
        L.enArrayQueue(q, src)
        # level 1 top-down, level 2 bottom-up, then top-down until empty
        L.topDownStepGraphCSR(g.ptr, q, None, stats)
        L.slideWindowArrayQueue(q)
        qq = q.contents
        for i in range(qq.head, qq.tail):
            L.setBit(cur, qq.queue[i])
        nf = L.bottomUpStepGraphCSR(g.ptr, cur, nxt, stats)
        assert nf == L.getNumOfSetBits(nxt)
        dist = np.ctypeslib.as_array(stats.contents.distances, shape=(g.V,)).copy()
        _, rd, _ = orc.bfs(o, 2, src)
        # vertices at levels <= 2 are exactly the reference's
        m = (rd <= 2) & ((rd > 0) | (np.arange(g.V) == src))
        np.testing.assert_array_equal(dist[m], rd[m])
        assert int(((dist > 0) & (dist <= 2)).sum()) == int(((rd > 0) & (rd <= 2)).sum())
    finally:
        L.freeArrayQueue(q)
        L.freeBitmap(cur)
        L.freeBitmap(nxt)
        L.freeBFSStats(stats)
        L.graphGpuRelease(g.ptr)
