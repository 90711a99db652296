"""CSR / CSC built on the GPU (gg_graph_build, graphCSRFromEdgeListDevice)
against the host build (graphCSRFromEdgeList), which sorts the same words
(row << b | neighbour) with a stable LSD radix sort: every array must be
identical — offsets, neighbour order within rows, the weights of duplicate
edges (input order), degrees, max_weight."""
import numpy as np
import pytest

from graphs import fixture_edges, special_edges

pytestmark = pytest.mark.gpu

KEYS = ("out_off", "out_adj", "in_off", "in_adj", "out_degree", "in_degree", "out_w", "in_w")


def _same(a, b, tag):
    for k in KEYS:
        if a[k] is None or b[k] is None:
            assert a[k] is None and b[k] is None, (tag, k)
            continue
        np.testing.assert_array_equal(a[k], b[k], err_msg=f"{tag} {k}")


def _cases():
    out = {}
    for name, (s, d, w) in fixture_edges().items():
        out[name] = (s, d, w, None)
    for name, (s, d, w, V) in special_edges().items():
        out[name] = (s, d, w, V)
    rng = np.random.default_rng(5)
    # duplicates of one edge with distinct weights: their order must be the input order
    s = rng.integers(0, 50, 4000).astype(np.uint32)
    d = rng.integers(0, 50, 4000).astype(np.uint32)
    out["dups_weighted"] = (s, d, rng.random(4000).astype(np.float32), 64)
    # vertex counts at and just past a power of two (the key width b changes)
    for V in (1, 2, 3, 255, 256, 257, 65536, 65537):
        E = 3 * V + 7
        out[f"rand_v{V}"] = (rng.integers(0, V, E).astype(np.uint32), rng.integers(0, V, E).astype(np.uint32),
                             rng.standard_normal(E).astype(np.float32), V)
    out["no_edges"] = (np.zeros(0, np.uint32), np.zeros(0, np.uint32), None, 10)
    return out


@pytest.mark.parametrize("name", sorted(_cases()))
def test_device_build_matches_host(gpu, name):
    s, d, w, V = _cases()[name]
    host = gpu.Graph.from_edges(s, d, w, num_vertices=V).arrays()
    dev_graph = gpu.Graph.from_edges(s, d, w, num_vertices=V, device_build=True)
    _same(dev_graph.arrays(), host, name)
    assert dev_graph.ptr.contents.max_weight == gpu.Graph.from_edges(s, d, w, num_vertices=V).ptr.contents.max_weight


@pytest.mark.parametrize("weighted", [False, True])
def test_device_build_rmat(gpu, weighted):
    """R-MAT scale 18 (262K vertices, 4.2M edges: several radix tiles per
    digit, skewed digits)."""
    host = gpu.Graph.rmat(18, 16, weighted=weighted).arrays()
    dev = gpu.Graph.rmat(18, 16, weighted=weighted, device_build=True).arrays()
    _same(dev, host, f"rmat18 weighted={weighted}")


def test_device_mapping_download(gpu):
    """gg_graph_build's mapping, downloaded, equals the host build; the
    mapping from device tensors equals the one from host arrays."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(9)
    V, E = 100_003, 1_500_000
    s = rng.integers(0, V, E).astype(np.uint32)
    d = (rng.zipf(1.6, E) % V).astype(np.uint32)
    w = rng.random(E).astype(np.float32)
    host = gpu.Graph.from_edges(s, d, w, num_vertices=V).arrays()
    dg = gpu.DeviceGraph.build(s, d, w, num_vertices=V)
    got = dg.download()
    for k in ("out_off", "out_adj", "in_off", "in_adj", "out_w", "in_w"):
        np.testing.assert_array_equal(got[k], host[k], err_msg=k)
    ts = torch.from_numpy(s.view(np.int32)).cuda()
    td = torch.from_numpy(d.view(np.int32)).cuda()
    tw = torch.from_numpy(w).cuda()
    dg2 = gpu.DeviceGraph.build(ts, td, tw, num_vertices=V)
    got2 = dg2.download()
    for k in ("out_off", "out_adj", "in_off", "in_adj", "out_w", "in_w"):
        np.testing.assert_array_equal(got2[k], host[k], err_msg="device input " + k)
    assert got2["max_weight"] == np.float32(w.max())


def test_device_built_mapping_runs_the_path(gpu, orc):
    """PageRank, SpMV and BFS on a mapping built on the device give the same
    results as on the host-built mapping of the same edges."""
    g = gpu.Graph.rmat(14, 16, weighted=True)
    a = g.arrays()
    s = np.repeat(np.arange(g.V, dtype=np.uint32), np.diff(a["out_off"]).astype(np.int64))
    dm = gpu.DeviceGraph.build(s, a["out_adj"], a["out_w"], num_vertices=g.V)
    hm = gpu.DeviceGraph(g, gpu.MAP_ALL)
    # the same arrays run the same kernels; rows split across tiles add FP32
    # partials with atomics, so sums may differ in the last bit
    r1, i1 = dm.pagerank("pull")
    r2, i2 = hm.pagerank("pull")
    np.testing.assert_allclose(r1, r2, rtol=1e-6, atol=0)
    assert i1["iterations"] == i2["iterations"]
    _, y1, _ = dm.spmv("pull")
    _, y2, _ = hm.spmv("pull")
    np.testing.assert_allclose(y1, y2, rtol=1e-6, atol=1e-30)
    _, d1, b1 = dm.bfs(0, "do")
    _, d2, b2 = hm.bfs(0, "do")
    np.testing.assert_array_equal(d1, d2)
    assert b1["edges_examined"] == b2["edges_examined"]


def test_device_build_rejects_bad_ids(gpu):
    s = np.array([0, 1, 7], np.uint32)
    d = np.array([1, 2, 3], np.uint32)
    with pytest.raises(gpu.GgError):
        gpu.DeviceGraph.build(s, d, num_vertices=5)


@pytest.mark.parametrize("route,misaligned", [("staged", False), ("driver", False), ("device", False),
                                              ("device", True)])
def test_copies_of_pageable_buffers(gpu, orc, route, misaligned):
    """Pageable host buffers above 4 MB, by each route of
    gg_set_host_copy_mode: page-locked staging in 32 MB chunks, the driver's
    pageable copy, and a kernel reading the source in place where the GPU
    uses the host's page tables (16-byte aligned sources only: the bytes past
    the last full 16 go by a small copy; an unaligned source is staged).  An
    80 MB edge list whose size is not a multiple of 16 bytes, uploaded by
    gg_graph_build (aligned, and 4 bytes off alignment), and 33.5 MB of BFS
    distances copied back into a numpy array arrive intact."""
    gpu.set_host_copy_mode(route)
    try:
        _pageable_case(gpu, orc, misaligned)
    finally:
        gpu.set_host_copy_mode("auto")


def _pageable_case(gpu, orc, misaligned):
    import ctypes as C

    rng = np.random.default_rng(12)
    V, E = 1 << 23, 20_000_001
    s = rng.integers(0, V, E).astype(np.uint32)
    d = rng.integers(0, V, E).astype(np.uint32)
    if misaligned:
        # the edge list's arrays (64-byte aligned, 64 bytes of slack) seen
        # from 4 bytes in; the original pointers are put back before freeing
        L = gpu.lib()
        el = gpu.Graph._edge_list(s, d, num_vertices=V)
        e = el.contents
        names = ("edges_array_src", "edges_array_dest")
        ptype = type(e.edges_array_src)
        # the addresses, not the field objects (those share the struct's memory)
        keep = [C.cast(getattr(e, n), C.c_void_p).value for n in names]
        try:
            for name, arr in (("edges_array_src", s), ("edges_array_dest", d)):
                addr = C.cast(getattr(e, name), C.c_void_p).value + 4
                assert addr % 16
                C.memmove(addr, arr.ctypes.data, E * 4)
                setattr(e, name, C.cast(C.c_void_p(addr), type(getattr(e, name))))
            dg = gpu.DeviceGraph.__new__(gpu.DeviceGraph)
            dg.h = C.c_void_p()
            st = L.gg_graph_build(el, gpu.MAP_OUT | gpu.MAP_IN, None, C.byref(dg.h))
            assert st == 0, L.gg_last_error().decode()
            dg.graph = gpu._Shape(V, E)
        finally:
            for n, addr in zip(names, keep):
                setattr(e, n, C.cast(C.c_void_p(addr), ptype))
            assert [C.cast(getattr(e, n), C.c_void_p).value for n in names] == keep
            L.freeEdgeList(el)
    else:
        dg = gpu.DeviceGraph.build(s, d, num_vertices=V, what=gpu.MAP_OUT | gpu.MAP_IN)
    got = dg.download(weights=False)
    host = gpu.Graph.from_edges(s, d, num_vertices=V).arrays()
    for k in ("out_off", "out_adj", "in_off", "in_adj"):
        np.testing.assert_array_equal(got[k], host[k], err_msg=k)
    src = int(s[0])
    _, dist, _ = dg.bfs(src, "push")
    g = gpu.Graph.from_edges(s, d, num_vertices=V)
    a = g.arrays()
    o = orc.Csr.from_arrays(V, E, a["out_off"], a["out_adj"], a["in_off"], a["in_adj"])
    _, rd, _ = orc.bfs(o, 1, src)
    np.testing.assert_array_equal(dist, rd)
