"""Degree-based relabelling (the reference's -l modes 0..10) on the GPU:
labels equal the oracle's restatement of each published algorithm (exact),
the relabelled CSR equals the host build of the relabelled edge list, and the
hot path's results map back through the labels (BFS levels and connected
components exactly, PageRank within FP32 rounding)."""
import os

import numpy as np
import pytest

from graphs import GOLDEN, fixture_edges, special_edges

pytestmark = pytest.mark.gpu

MODES = list(range(11))


def _edge_sets(orc):
    out = {}
    for name, (s, d, w) in fixture_edges().items():
        out[name] = (s, d, w, int(max(s.max(), d.max())) + 1)
    for name, (s, d, w, V) in special_edges().items():
        out[name] = (s, d, w, V)
    s, d, w = orc.rmat_edges(14, 8, weighted=True)
    out["rmat14"] = (s, d, w, 1 << 14)
    s, d, _ = orc.rmat_edges(12, 4, symmetric=True)
    out["rmat12u"] = (s, d, None, 1 << 12)
    return out


@pytest.mark.parametrize("lmode", MODES)
def test_relabel_order_matches_oracle(gpu, orc, lmode):
    for name, (s, d, w, V) in _edge_sets(orc).items():
        got = gpu.relabel_order(s, d, V, lmode, seed=123)
        want = orc.relabel_order(s, d, V, lmode, seed=123)
        np.testing.assert_array_equal(got, want, err_msg=f"{name} mode {lmode}")
        assert np.array_equal(np.sort(got), np.arange(V, dtype=np.uint32))


@pytest.mark.parametrize("lmode", [1, 4, 7, 8, 10])
def test_relabelled_csr_equals_host_build(gpu, orc, lmode):
    for name in ("v300_e2730", "rmat14", "hubs"):
        s, d, w, V = _edge_sets(orc)[name]
        g = gpu.Graph.from_edges_relabelled(s, d, w, num_vertices=V, lmode=lmode, seed=7)
        label, inverse = g.labels()
        want = orc.relabel_order(s, d, V, lmode, seed=7)
        np.testing.assert_array_equal(label, want)
        np.testing.assert_array_equal(inverse[label], np.arange(V, dtype=np.uint32))
        host = gpu.Graph.from_edges(label[s], label[d], w, num_vertices=V).arrays()
        a = g.arrays()
        for k in ("out_off", "out_adj", "in_off", "in_adj", "out_w", "in_w", "out_degree", "in_degree"):
            if host[k] is None:
                assert a[k] is None
            else:
                np.testing.assert_array_equal(a[k], host[k], err_msg=f"{name} {k}")


def test_results_map_back_through_labels(gpu, orc):
    s, d, w, V = _edge_sets(orc)["rmat14"]
    g0 = gpu.Graph.from_edges(s, d, w, num_vertices=V)
    g1 = gpu.Graph.from_edges_relabelled(s, d, w, num_vertices=V, lmode=5)
    label, _ = g1.labels()
    d0 = gpu.DeviceGraph(g0, gpu.MAP_ALL)
    d1 = gpu.DeviceGraph(g1, gpu.MAP_ALL)
    # BFS levels: exact
    deg = np.bincount(s, minlength=V)
    for src in np.flatnonzero(deg)[:5]:
        _, dist0, r0 = d0.bfs(int(src), "do")
        _, dist1, r1 = d1.bfs(int(label[src]), "do")
        np.testing.assert_array_equal(dist1[label], dist0)
        assert r0["processed_nodes"] == r1["processed_nodes"]
    # connected components: the same partition
    c0, _ = d0.cc("afforest")
    c1, _ = d1.cc("afforest")
    inv = np.empty(V, np.uint32)
    inv[label] = np.arange(V, dtype=np.uint32)
    back = c1[label]  # component of each original vertex, as a relabelled id
    mins = np.full(V, V, np.int64)
    np.minimum.at(mins, back, np.arange(V))
    np.testing.assert_array_equal(mins[back].astype(np.uint32), c0)
    # PageRank: the same ranks up to FP32 summation order
    r0, i0 = d0.pagerank("pull", iterations=20, epsilon=0.0)
    r1, i1 = d1.pagerank("pull", iterations=20, epsilon=0.0)
    np.testing.assert_allclose(r1[label], r0, rtol=2e-5, atol=1e-12)


def test_relabel_from_file_labels_and_bad_permutation(gpu, orc):
    """Mode 11 (labels from a file): any permutation builds the permuted
    graph; an array that is not a permutation is rejected."""
    s, d, w, V = _edge_sets(orc)["rmat14"]
    rng = np.random.default_rng(3)
    label = rng.permutation(V).astype(np.uint32)
    dg = gpu.build_relabelled(s, d, label, w, num_vertices=V)
    got = dg.download()
    host = gpu.Graph.from_edges(label[s], label[d], w, num_vertices=V).arrays()
    for k in ("out_off", "out_adj", "in_off", "in_adj", "out_w", "in_w"):
        np.testing.assert_array_equal(got[k], host[k], err_msg=k)
    bad = label.copy()
    bad[0] = bad[1]
    with pytest.raises(gpu.GgError):
        gpu.build_relabelled(s, d, bad, w, num_vertices=V)
    with pytest.raises(gpu.GgError):
        gpu.relabel_order(s, d, V, 12)
