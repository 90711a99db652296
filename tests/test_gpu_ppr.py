"""Batched personalised PageRank (gg_ppr) against the FP64 oracle.

Each of the K vectors is the pull PageRank of pageRank.c:1026-1069 with the
teleport going to its seed set; the oracle runs every vector on its own in
FP64 (orc_ppr_f64_multi) with the same damping factor as a float32.  FP32
storage must stay within L1 <= 1e-6 of FP64 per vector; BF16 storage within
the bound written below.  A vector's result must not depend on the vectors
batched with it.
"""
import numpy as np
import pytest

from graphs import pair, special_edges

pytestmark = pytest.mark.gpu

DAMP = float(np.float32(0.85))
ITERS = 20


@pytest.fixture(scope="module")
def rg(gpu, orc):
    return pair(gpu, orc, gpu.Graph.rmat(13, 16))


@pytest.fixture(scope="module")
def hub(gpu, orc):
    src, dst, w, V = special_edges()["hubs"]
    return pair(gpu, orc, gpu.Graph.from_edges(src, dst, w, num_vertices=V))


def seed_sets(V, K, deg, rng):
    """K seed sets of 1-8 vertices, with a repeated seed, a seed of out-degree
    0 (when the graph has one) and, for K > 4, one empty set."""
    sets = []
    zero = np.flatnonzero(deg == 0)
    for k in range(K):
        n = int(rng.integers(1, 9))
        s = list(rng.integers(0, V, n))
        if k == 1:
            s = s + [s[0]]
        if k == 2 and len(zero):
            s = [int(zero[0])]
        sets.append(s)
    if K > 4:
        sets[3] = []
    return sets


def oracle_vectors(orc, o, sets):
    out = []
    for s in sets:
        out.append(np.zeros(o.V) if not s else orc.ppr_f64_multi(o, s, ITERS, DAMP))
    return np.stack(out, 1)


@pytest.mark.parametrize("K", [3, 20, 64])
def test_ppr_f32_matches_fp64(gpu, orc, rg, K):
    g, o = rg
    rng = np.random.default_rng(K)
    sets = seed_sets(g.V, K, g.arrays()["out_degree"], rng)
    dg = gpu.DeviceGraph(g, gpu.MAP_IN)
    ranks, res = dg.ppr(sets, iterations=ITERS, storage="f32")
    dg.free()
    assert res["padded_vectors"] == (16 if K <= 16 else 32 if K <= 32 else 64)
    ex = oracle_vectors(orc, o, sets)
    l1 = np.abs(ranks - ex).sum(0)
    assert l1.max() <= 1e-6, l1
    if K > 4:
        assert not ranks[:, 3].any()


def test_ppr_bf16_bound(gpu, orc, rg):
    g, o = rg
    sets = seed_sets(g.V, 64, g.arrays()["out_degree"], np.random.default_rng(11))
    dg = gpu.DeviceGraph(g, gpu.MAP_IN)
    ranks, _ = dg.ppr(sets, iterations=ITERS, storage="bf16")
    dg.free()
    ex = oracle_vectors(orc, o, sets)
    l1 = np.abs(ranks - ex).sum(0)
    mass = np.abs(ex).sum(0)
    # BF16 keeps 8 significant bits per stored contribution (rounding error
    # up to 2^-9 relative), summed in FP32.  Each iteration's rounding is
    # contracted by d per later iteration, so the error settles near
    # 2^-9 / (1 - d) times the mass with random signs: a numpy restatement
    # of this storage over 320 seed sets drawn as here on R-MAT-13 gives at
    # most 4.1e-3 of a vector's mass (a small set concentrates its mass on
    # few rows), and R-MAT-22 measures 3.0e-3.  Bound: 8e-3.  (Storing
    # BF16 deltas with an FP32 stored-so-far value -- the PageRank correction
    # pass -- only reaches ~1e-4 here: a PPR vector's change per iteration
    # decays like d^t, so every iteration's rounding weighs the same.)
    assert (l1 <= 8e-3 * np.maximum(mass, 1e-30)).all(), (l1 / np.maximum(mass, 1e-30)).max()


def test_ppr_hub_rows_span_tiles(gpu, orc, hub):
    g, o = hub
    sets = [[0], [3], [3, 0, 150], list(range(100, 140))]
    dg = gpu.DeviceGraph(g, gpu.MAP_IN)
    ranks, _ = dg.ppr(sets, iterations=ITERS, storage="f32")
    dg.free()
    ex = oracle_vectors(orc, o, sets)
    # vertex 0 sums 9000 in-edges in FP32 (relative error up to n*2^-24,
    # ~5e-6 seen); every other row is within the R-MAT bound
    err = np.abs(ranks - ex)
    assert err.sum(0).max() <= 1e-5
    assert err[1:].sum(0).max() <= 1e-6


@pytest.mark.parametrize("storage", ["f32", "bf16"])
def test_ppr_vector_independent_of_batch(gpu, rg, storage):
    """A vector's result is bit-identical alone, in a batch of 64 and in the
    same batch reordered: each vector's sums run in CSC edge order and rows
    spanning tiles add their per-tile partials in tile order."""
    g, _ = rg
    sets = seed_sets(g.V, 64, g.arrays()["out_degree"], np.random.default_rng(3))
    dg = gpu.DeviceGraph(g, gpu.MAP_IN)
    batch, _ = dg.ppr(sets, iterations=ITERS, storage=storage)
    perm = np.random.default_rng(4).permutation(64)
    shuffled, _ = dg.ppr([sets[i] for i in perm], iterations=ITERS, storage=storage)
    np.testing.assert_array_equal(shuffled, batch[:, perm])
    for k in (0, 1, 2, 40, 63):
        alone, _ = dg.ppr([sets[k]], iterations=ITERS, storage=storage)
        np.testing.assert_array_equal(alone[:, 0], batch[:, k])
    dg.free()


def test_ppr_rejects_bad_arguments(gpu, rg):
    g, _ = rg
    dg = gpu.DeviceGraph(g, gpu.MAP_IN)
    with pytest.raises(gpu.GgError):
        dg.ppr([[0]] * 65)
    with pytest.raises(gpu.GgError):
        dg.ppr([[g.V]])
    with pytest.raises(gpu.GgError):
        dg.ppr([[0]], iterations=0)
    with pytest.raises(gpu.GgError):
        dg.ppr([[0]], storage="f16")
    dg.free()


def test_ppr_persistent_launch_equals_per_iteration_launches(gpu, rg):
    """gg_ppr runs every iteration in one cooperative launch (grid barriers
    between the gather and the fix-up of the rows spanning tiles); with
    profile on it launches the two phases per iteration instead.  Same
    arithmetic in the same order: bit-identical results."""
    g, _ = rg
    sets = seed_sets(g.V, 40, g.arrays()["out_degree"], np.random.default_rng(8))
    dg = gpu.DeviceGraph(g, gpu.MAP_IN)
    for storage in ("f32", "bf16"):
        one, r1 = dg.ppr(sets, iterations=ITERS, storage=storage)
        many, r2 = dg.ppr(sets, iterations=ITERS, storage=storage, profile=True)
        # seed contributions, 1 / out-degree, the persistent launch (and the
        # tile coordinates on a mapping's first call)
        assert r1["persistent"] == 1 and r1["launches"] <= 4
        assert r2["persistent"] == 0 and r2["gather_launches"] == ITERS
        np.testing.assert_array_equal(one, many)
    dg.free()


def test_ppr_barrier_wait_runs_out_and_the_context_recovers(gpu, rg):
    """A grid-barrier wait limit of 1 us runs out while the blocks with
    tiles are still gathering: the launch ends, gg_ppr reports a kernel
    error, and the next call (default limit) gives the same ranks as
    before, on the same context."""
    g, _ = rg
    sets = seed_sets(g.V, 16, g.arrays()["out_degree"], np.random.default_rng(9))
    dg = gpu.DeviceGraph(g, gpu.MAP_IN)
    good, _ = dg.ppr(sets, iterations=ITERS, storage="f32")
    L = gpu.lib()
    L.gg_set_barrier_limit_us(1)
    try:
        with pytest.raises(gpu.GgError, match="timed out"):
            dg.ppr(sets, iterations=ITERS, storage="f32")
    finally:
        L.gg_set_barrier_limit_us(0)
    again, _ = dg.ppr(sets, iterations=ITERS, storage="f32")
    np.testing.assert_array_equal(again, good)
    dg.free()
