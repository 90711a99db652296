"""The autotuner (gg_autotune): it times candidate launch shapes on a
mapping, keeps the fastest, and remembers it for graphs of the same class.

* On R-MAT-16, -20 and -24 the PageRank pull gather in the tuned shape is at
  least as fast as in the default shape (re-measured after tuning, median of
  seven gather launches each, 5% allowance for run-to-run noise), and the
  ranks stay within the floating-point rule against the FP64 oracle.
* A second mapping of the same graph starts with the remembered shape; the
  picks survive gg_tune_save / gg_tune_reset / gg_tune_load.
* BFS, batched PPR and the many-graphs batch tune to valid shapes whose
  results are unchanged (BFS levels exact, PPR and batch within their rules).
"""
import numpy as np
import pytest

from fpcheck import assert_fp_as_accurate

pytestmark = pytest.mark.gpu


def _gather_ms(dg, n=7, storage="f32"):
    t = []
    for _ in range(n):
        _, r = dg.pagerank("pull", storage=storage, iterations=3, epsilon=0.0, copy_out=False, profile=True)
        t.append(r["gather_ms"] / max(r["gather_launches"], 1))
    return float(np.median(t))


@pytest.mark.parametrize("scale", [16, 20, 24])
def test_tuned_pagerank_gather_not_slower_than_default(gpu, orc, scale):
    gpu.tune_reset()
    g = gpu.Graph.rmat(scale, 16)
    tuned = gpu.DeviceGraph(g, gpu.MAP_IN)
    picks = tuned.autotune(gpu.TUNE_PR, reps=3)
    assert "pr" in picks and picks["pr"]["candidates"] >= 6
    assert picks["pr"]["tuned_ms"] <= picks["pr"]["default_ms"]
    gpu.tune_reset()  # the default mapping must not pick the shape up
    plain = gpu.DeviceGraph(g, gpu.MAP_IN)
    t_default = _gather_ms(plain)
    t_tuned = _gather_ms(tuned)
    assert t_tuned <= 1.05 * t_default, (picks, t_tuned, t_default)
    if scale == 16:
        a = g.arrays()
        o = orc.Csr.from_arrays(g.V, g.E, a["out_off"], a["out_adj"], a["in_off"], a["in_adj"])
        ranks, res = tuned.pagerank("pull", iterations=20, epsilon=1e-4)
        ref, info = orc.pagerank(o, 0, 20, 1e-4)
        assert res["iterations"] == info["iterations"]
        assert_fp_as_accurate(ranks, ref, orc.pagerank_f64(o, info["executed"]), "tuned shape")
    tuned.free()
    plain.free()
    g.free()


def test_remembered_shapes_reach_new_mappings_and_files(gpu, tmp_path):
    gpu.tune_reset()
    g = gpu.Graph.rmat(18, 16)
    a = gpu.DeviceGraph(g, gpu.MAP_IN)
    a.autotune(gpu.TUNE_PR, reps=2)
    pick = a.tuned(gpu.TUNE_PR)
    b = gpu.DeviceGraph(g, gpu.MAP_IN)
    b.pagerank("pull", iterations=1, epsilon=0.0, copy_out=False)  # first call: the lookup
    assert b.tuned(gpu.TUNE_PR) == pick
    path = str(tmp_path / "tune.txt")
    gpu.tune_save(path)
    gpu.tune_reset()
    c = gpu.DeviceGraph(g, gpu.MAP_IN)
    c.pagerank("pull", iterations=1, epsilon=0.0, copy_out=False)
    assert c.tuned(gpu.TUNE_PR) == [2, 5, 32, 0, 0]  # the default, nothing remembered
    gpu.tune_load(path)
    d = gpu.DeviceGraph(g, gpu.MAP_IN)
    d.pagerank("pull", iterations=1, epsilon=0.0, copy_out=False)
    assert d.tuned(gpu.TUNE_PR) == pick
    for x in (a, b, c, d):
        x.free()
    g.free()
    gpu.tune_reset()


def test_bfs_and_ppr_tuning_keep_results(gpu, orc):
    gpu.tune_reset()
    g = gpu.Graph.rmat(16, 16, symmetric=True)
    a = g.arrays()
    o = orc.Csr.from_arrays(g.V, g.E, a["out_off"], a["out_adj"], a["in_off"], a["in_adj"])
    dg = gpu.DeviceGraph(g, gpu.MAP_IN | gpu.MAP_OUT)
    before, _ = dg.ppr([[1], [2, 3]], iterations=10, storage="f32")
    picks = dg.autotune(gpu.TUNE_BFS | gpu.TUNE_PPR, reps=2)
    assert picks["bfs"]["params"][0] in (32, 64, 128, 256, 1024)
    assert picks["ppr"]["params"][0] in (256, 512, 1024)
    deg = np.diff(o.out_off.astype(np.int64))
    for s in np.nonzero(deg)[0][:6]:
        _, dist, res = dg.bfs(int(s), "do")
        _, rd, info = orc.bfs(o, 2, int(s))
        np.testing.assert_array_equal(dist, rd)
        assert res["edges_examined"] == info["edges_examined"]
    after, _ = dg.ppr([[1], [2, 3]], iterations=10, storage="f32")
    # another tile size changes which rows span tiles, not the FP64 answer
    ex = np.stack([orc.ppr_f64_multi(o, s, 10, float(np.float32(0.85))) for s in ([1], [2, 3])], 1)
    assert np.abs(after - ex).sum(0).max() <= 1e-6
    assert np.abs(before - ex).sum(0).max() <= 1e-6
    dg.free()
    g.free()
    gpu.tune_reset()


def test_batch_tuning_picks_a_valid_shape(gpu, orc):
    gpu.tune_reset()
    scales = [5, 9, 7, 10, 6, 8, 11, 12]
    g, voff = gpu.Graph.rmat_batch(scales, edge_factor=8, seed0=77)
    dg = gpu.DeviceGraph(g, gpu.MAP_IN)
    picks = dg.autotune(gpu.TUNE_BATCH, reps=2, vertex_off=voff)
    ipt, warps, vmax, ctas, strategy = picks["batch"]["params"]
    assert ipt in (5, 7, 9) and warps in (4, 8, 16, 32) and ctas in (1, 2, 4, 8) and strategy in (1, 2)
    assert picks["batch"]["tuned_ms"] <= picks["batch"]["default_ms"]
    assert dg.tuned(gpu.TUNE_BATCH) == [ipt, warps, vmax, ctas, strategy]
    ranks, _ = dg.pagerank_batch(voff, iterations=20, epsilon=0.0)
    for i, sc in enumerate(scales):
        o = orc.rmat_csr(sc, 8, seed=77 + i)
        ref, info = orc.pagerank(o, 0, 20, 0.0)
        assert_fp_as_accurate(ranks[voff[i]:voff[i + 1]], ref, orc.pagerank_f64(o, 20), f"graph {i}")
    dg.free()
    g.free()
    gpu.tune_reset()
