"""BFS on the GPU vs the oracle and the reference's golden vectors.

Bit-exact: distances (levels), processed_nodes and the reference's
`iteration` count, for every mode and source.  Parents found top-down depend
on which CAS wins (they do in the reference too), so they are checked
structurally (parent one level up, edge parent -> vertex); the all-bottom-up
pull mode takes the first in-neighbour in CSC order and is bit-exact.
"""
import os

import numpy as np
import pytest

from graphs import GOLDEN, fixture_edges, pair, special_edges

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def graphs(gpu, orc):
    out = {}
    for name, (s, d, w) in fixture_edges().items():
        out[name] = pair(gpu, orc, gpu.Graph.from_edges(s, d, w))
    for name, (s, d, w, V) in special_edges().items():
        out[name] = pair(gpu, orc, gpu.Graph.from_edges(s, d, w, num_vertices=V))
    out["rmat8"] = pair(gpu, orc, gpu.Graph.rmat(8, 8, weighted=True))
    out["rmat10"] = pair(gpu, orc, gpu.Graph.rmat(10, 16, weighted=True))
    out["rmat12u"] = pair(gpu, orc, gpu.Graph.rmat(12, 8, weighted=True, symmetric=True))
    out["rmat16u"] = pair(gpu, orc, gpu.Graph.rmat(16, 16, symmetric=True))
    out["rmat16"] = pair(gpu, orc, gpu.Graph.rmat(16, 16))
    return out


@pytest.fixture(scope="module")
def dgs(gpu, graphs):
    return {k: gpu.DeviceGraph(g, gpu.MAP_ALL) for k, (g, _) in graphs.items()}


def _sources(V):
    return sorted({0, 1, V // 2, V - 1} & set(range(V)))


@pytest.mark.parametrize("mode", list(range(5)))
def test_bfs_modes_vs_oracle(graphs, dgs, orc, mode):
    for name, (g, o) in graphs.items():
        for s in _sources(g.V):
            parents, dist, res = dgs[name].bfs(s, mode)
            rp, rd, info = orc.bfs(o, mode, s)
            tag = f"{name} mode {mode} source {s}"
            np.testing.assert_array_equal(dist, rd, err_msg=tag)
            assert res["processed_nodes"] == info["processed_nodes"], tag
            assert 1 + res["levels"] == info["iteration"], tag
            assert res["top_down_steps"] == info["top_down_steps"], tag
            assert res["bottom_up_steps"] == info["bottom_up_steps"], tag
            if mode == 0:
                np.testing.assert_array_equal(parents, rp, err_msg=tag)
            else:
                levels = orc.bfs_levels_reference(o, s)
                orc.check_parents(o, s, parents, levels)
                # levels of reached vertices equal distances; unreached keep 0
                assert np.array_equal(np.where(levels >= 0, levels, 0), dist), tag


@pytest.mark.parametrize("name", ["graphbrew", "test", "v51_e1021", "v300_e2730", "rmat8", "rmat10", "rmat12u",
                                  "hubs", "single", "star_out", "star_in", "ring", "no_edges"])
def test_bfs_vs_reference_golden(graphs, dgs, name):
    """Against the reference's own BFS.c (tests/golden)."""
    z = np.load(os.path.join(GOLDEN, f"golden_{name}.npz"))
    g, o = graphs[name]
    for mode in range(5):
        for s in z["bfs_sources"]:
            s = int(s)
            parents, dist, res = dgs[name].bfs(s, mode)
            tag = f"{name} mode {mode} source {s}"
            np.testing.assert_array_equal(dist, z[f"bfs{mode}_{s}_dist"], err_msg=tag)
            assert res["processed_nodes"] == int(z[f"bfs{mode}_{s}_processed"]), tag
            assert 1 + res["levels"] == int(z[f"bfs{mode}_{s}_iteration"]), tag
            if mode == 0:
                np.testing.assert_array_equal(parents, z[f"bfs{mode}_{s}_parents"], err_msg=tag)
            rp = z[f"bfs{mode}_{s}_parents"]
            np.testing.assert_array_equal(parents < 0, rp < 0, err_msg=tag)
            np.testing.assert_array_equal(parents[rp < 0], rp[rp < 0], err_msg=tag)


def test_bfs_many_sources_rmat16(graphs, dgs, orc):
    g, o = graphs["rmat16u"]
    rng = np.random.default_rng(3)
    deg = np.diff(o.out_off.astype(np.int64))
    cand = np.nonzero(deg)[0]
    for s in rng.choice(cand, 16, replace=False):
        _, dist, res = dgs["rmat16u"].bfs(int(s), "do")
        _, rd, info = orc.bfs(o, 2, int(s))
        np.testing.assert_array_equal(dist, rd)
        assert res["edges_examined"] == info["edges_examined"]


def test_bfs_invalid_source(gpu, dgs):
    with pytest.raises(gpu.GgError):
        dgs["rmat8"].bfs(256, "do")


@pytest.mark.parametrize("mode", ["do", 4])
def test_bfs_device_loop_matches_host_loop(graphs, dgs, mode):
    """The direction-optimised modes run their level loop in one cooperative
    launch unless profiled; profiled searches step from the host.  Both must
    give the same schedule, counts and levels."""
    rng = np.random.default_rng(11)
    for name in ("rmat12u", "rmat16u", "rmat16", "rmat10"):
        g, o = graphs[name]
        deg = np.diff(o.out_off.astype(np.int64))
        cand = np.nonzero(deg)[0]
        for s in list(rng.choice(cand, 6, replace=False)) + [0]:
            _, d0, r0 = dgs[name].bfs(int(s), mode, profile=False)
            _, d1, r1 = dgs[name].bfs(int(s), mode, profile=True)
            tag = f"{name} source {s}"
            np.testing.assert_array_equal(d0, d1, err_msg=tag)
            for k in ("processed_nodes", "levels", "top_down_steps", "bottom_up_steps", "edges_examined"):
                assert r0[k] == r1[k], (tag, k, r0[k], r1[k])
            assert r0["launches"] == 2, (tag, r0["launches"])  # k_bfs_init and k_bfs_do


def test_bfs_barrier_wait_runs_out_and_the_context_recovers(gpu, graphs, dgs, orc):
    """The single-launch direction-optimising search waits at grid barriers
    with a device-side limit.  At 1 us the blocks that reach a barrier first
    give up while the others are still working: the search ends early and
    gg_bfs reports a kernel error.  The next search, at the default limit,
    is exact against the oracle on the same context."""
    g, o = graphs["rmat16u"]
    s = int(np.nonzero(np.diff(o.out_off.astype(np.int64)))[0][0])
    L = gpu.lib()
    L.gg_set_barrier_limit_us(1)
    try:
        with pytest.raises(gpu.GgError, match="timed out"):
            dgs["rmat16u"].bfs(s, "do")
    finally:
        L.gg_set_barrier_limit_us(0)
    _, dist, res = dgs["rmat16u"].bfs(s, "do")
    _, rd, info = orc.bfs(o, 2, s)
    np.testing.assert_array_equal(dist, rd)
    assert res["edges_examined"] == info["edges_examined"]


def test_host_wait_limit_returns_timeout_and_work_completes(gpu, graphs, dgs, orc):
    """Every host wait on device work polls with a limit
    (gg_set_wait_timeout_ms).  A 1 ms limit on a PageRank that runs longer
    returns GG_ETIMEDOUT (5) instead of blocking; the queued work still
    completes, and a call at the default limit is correct."""
    import ctypes as C

    L = gpu.lib()
    big = gpu.Graph.rmat(20, 16)
    d = gpu.DeviceGraph(big, gpu.MAP_IN)
    d.pagerank("pull", iterations=2, epsilon=0.0)  # tiles and work buffers exist
    p = gpu.PrParams(0, 0, 200, 0, 0.0, 0.85, 0, 0x2)  # 200 FP32 pull iterations, hot table off
    r = gpu.PrResult()
    L.gg_set_wait_timeout_ms(1)
    try:
        st = L.gg_pagerank(d.h, C.byref(p), None, C.byref(r), None)
    finally:
        L.gg_set_wait_timeout_ms(0)
    assert st == 5, (st, L.gg_last_error())
    g, o = graphs["rmat16"]
    ranks, res = dgs["rmat16"].pagerank("pull", iterations=20, epsilon=1e-4)
    ref, info = orc.pagerank(o, 0, 20, 1e-4)
    assert res["iterations"] == info["iterations"]
    d.pagerank("pull", iterations=2, epsilon=0.0)  # waits behind the 200 iterations
    d.free()
    big.free()
