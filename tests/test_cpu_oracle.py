"""The oracle, pinned: against the golden vectors made by the reference's own
code (tests/golden), and -- where the reference tree is mounted -- against
that code live.  Runs on CPU."""
import os

import numpy as np
import pytest

from graphs import GOLDEN, fixture_edges, special_edges

SPECIAL = ["hubs", "single", "star_out", "star_in", "ring", "no_edges"]
NAMES = ["graphbrew", "test", "v51_e1021", "v300_e2730", "rmat8", "rmat10", "rmat12u"] + SPECIAL
RMAT = {"rmat8": (8, 8, False), "rmat10": (10, 16, False), "rmat12u": (12, 8, True)}


def _graph(orc, name, weighted=True):
    if name in RMAT:
        s, e, sym = RMAT[name]
        src, dst, w = orc.rmat_edges(s, e, weighted=weighted, symmetric=sym)
        return orc.Csr(1 << s, src, dst, w)
    if name in SPECIAL:
        src, dst, w, V = special_edges()[name]
        return orc.Csr(V, src, dst, w if weighted else None)
    src, dst, w = fixture_edges()[name]
    V = int(max(src.max(), dst.max())) + 1
    return orc.Csr(V, src, dst, w if weighted else None)


@pytest.mark.parametrize("name", NAMES)
def test_oracle_pagerank_matches_reference_golden(orc, name):
    z = np.load(os.path.join(GOLDEN, f"golden_{name}.npz"))
    g = _graph(orc, name)
    for mode in range(14):
        r, info = orc.pagerank(g, mode, 20, 1e-4)
        np.testing.assert_array_equal(r.view(np.uint32), z[f"pr{mode}_ranks"].view(np.uint32),
                                      err_msg=f"{name} mode {mode}")
        assert info["iterations"] == int(z[f"pr{mode}_iters"])
        assert info["error_total"] == float(z[f"pr{mode}_err"])


@pytest.mark.parametrize("name", NAMES)
def test_oracle_bfs_matches_reference_golden(orc, name):
    z = np.load(os.path.join(GOLDEN, f"golden_{name}.npz"))
    g = _graph(orc, name)
    for mode in range(5):
        for s in z["bfs_sources"]:
            s = int(s)
            p, d, info = orc.bfs(g, mode, s)
            np.testing.assert_array_equal(p, z[f"bfs{mode}_{s}_parents"])
            np.testing.assert_array_equal(d, z[f"bfs{mode}_{s}_dist"])
            assert info["processed_nodes"] == int(z[f"bfs{mode}_{s}_processed"])
            assert info["iteration"] == int(z[f"bfs{mode}_{s}_iteration"])


@pytest.mark.parametrize("name", NAMES)
def test_oracle_spmv_matches_reference_golden(orc, name):
    z = np.load(os.path.join(GOLDEN, f"golden_{name}.npz"))
    g = _graph(orc, name, weighted=False)
    for mode in (0, 1, 3):
        x, y, _ = orc.spmv(g, mode, 3)
        np.testing.assert_array_equal(x, z[f"spmv{mode}_x"])
        np.testing.assert_array_equal(y.view(np.uint32), z[f"spmv{mode}_y"].view(np.uint32))
    # the reference's pull fixed-point variant returns zeros (SPMV.c:980-983)
    assert not z["spmv2_y"].any()


@pytest.mark.parametrize("name", NAMES)
def test_oracle_cc_matches_reference_golden(orc, name):
    """The reference's own connectedComponents.c (Afforest and weakly, run
    by tests/golden/make_golden.py): its labels are the oracle's, and its
    stats arrays are the component sizes sorted ascending with the label of
    each beside it (ties in ascending id); its Afforest counts no
    iterations."""
    z = np.load(os.path.join(GOLDEN, f"golden_{name}.npz"))
    want = orc.cc_min_label(_graph(orc, name))
    size = np.bincount(want, minlength=len(want)).astype(np.uint32)
    order = np.argsort(size, kind="stable").astype(np.uint32)
    for mode in (1, 2):
        np.testing.assert_array_equal(z[f"cc{mode}_components"], want, err_msg=f"{name} {mode}")
        np.testing.assert_array_equal(z[f"cc{mode}_labels"], order, err_msg=f"{name} {mode}")
        np.testing.assert_array_equal(z[f"cc{mode}_counts"], size[order], err_msg=f"{name} {mode}")
    assert int(z["cc1_iterations"]) == 0


def test_sample_frequent_node_as_the_reference(gg, orc):
    """The drop-in's sampleFrequentNode against the reference's own
    (connectedComponents.c:293-334): same label, ties to the smallest, and
    the caller's generator left in the same state."""
    import ctypes as C

    R = orc.ref_lib()
    if R is None:
        pytest.skip("reference tree not mounted here")
    L = gg.lib()
    rng = np.random.default_rng(3)
    cases = [(1000, 500, rng.integers(0, 7, 1000)), (5000, 1024, rng.integers(0, 5000, 5000)),
             (16, 64, np.arange(16)), (9, 3, np.arange(9))]
    for V, S, comp in cases:
        comp = np.ascontiguousarray(comp, np.uint32)
        a, b = gg.default_arguments(), gg.default_arguments()
        got = L.sampleFrequentNode(C.byref(a.mt19937var), V, S, comp.ctypes.data_as(C.c_void_p))
        want = R.sampleFrequentNode(C.byref(b.mt19937var), V, S, comp.ctypes.data_as(C.c_void_p))
        R.ref_cc_reset()
        assert got == want, (V, S, got, want)
        assert bytes(a.mt19937var) == bytes(b.mt19937var), (V, S)


def test_host_helpers_as_the_reference(gg, orc):
    """The drop-in's host helpers against the reference's own, on the same
    inputs in one thread: the atomic adds and set of pageRank.c:188-252 and
    the minimum, link and compress of connectedComponents.c:233-283."""
    import ctypes as C

    R = orc.ref_lib()
    if R is None:
        pytest.skip("reference tree not mounted here")
    L = gg.lib()
    for lib in (L, R):
        lib.addAtomicFloat.argtypes = [C.POINTER(C.c_float), C.c_float]
        lib.addAtomicDouble.argtypes = [C.POINTER(C.c_double), C.c_double]
        lib.addAtomicFixedPoint.argtypes = [C.POINTER(C.c_uint64), C.c_uint64]
        lib.setAtomic.argtypes = [C.POINTER(C.c_uint64), C.c_uint64]
        lib.atomicMin.argtypes = [C.POINTER(C.c_uint32), C.c_uint32]
        lib.atomicMin.restype = C.c_uint32
        lib.linkNodes.argtypes = [C.c_uint32, C.c_uint32, C.c_void_p]
        lib.compressNodes.argtypes = [C.c_uint32, C.c_void_p]
    rng = np.random.default_rng(8)
    vals = rng.random(200)
    f = [C.c_float(0.125), C.c_float(0.125)]
    d = [C.c_double(0.125), C.c_double(0.125)]
    u = [C.c_uint64(3), C.c_uint64(3)]
    for v in vals:
        for k, lib in enumerate((L, R)):
            lib.addAtomicFloat(C.byref(f[k]), float(v))
            lib.addAtomicDouble(C.byref(d[k]), float(v))
            lib.addAtomicFixedPoint(C.byref(u[k]), int(v * 2**32))
    assert f[0].value == f[1].value and d[0].value == d[1].value and u[0].value == u[1].value
    for k, lib in enumerate((L, R)):
        lib.setAtomic(C.byref(u[k]), 12345)
    assert u[0].value == u[1].value == 12345
    for x, y in ((10, 3), (10, 12), (5, 5), (0, 7)):
        a, b = C.c_uint32(x), C.c_uint32(x)
        assert L.atomicMin(C.byref(a), y) == R.atomicMin(C.byref(b), y) and a.value == b.value
    V = 700
    src = rng.integers(0, V, 900)
    dst = rng.integers(0, V, 900)
    comps = [np.arange(V, dtype=np.uint32), np.arange(V, dtype=np.uint32)]
    for k, lib in enumerate((L, R)):
        for x, y in zip(src, dst):
            lib.linkNodes(int(x), int(y), comps[k].ctypes.data)
        lib.compressNodes(V, comps[k].ctypes.data)
    np.testing.assert_array_equal(comps[0], comps[1])


def test_print_cc_stats_fills_as_the_reference(gg, orc, capfd):
    """The same labelling through the reference's own printCCStats and the
    drop-in's: the same counts and labels arrays (both structs start as the
    reference's constructor leaves them: counts 0, labels the identity)."""
    import ctypes as C

    R = orc.ref_lib()
    if R is None:
        pytest.skip("reference tree not mounted here")
    L = gg.lib()
    rng = np.random.default_rng(12)
    for V in (1, 9, 500, 4000):
        comp = np.minimum.accumulate(rng.integers(0, V, V)).astype(np.uint32)  # labels that are vertex ids
        comp = np.where(rng.random(V) < 0.5, comp, np.arange(V, dtype=np.uint32)).astype(np.uint32)
        out = []
        for lib in (R, L):
            c = comp.copy()
            counts = np.zeros(V, np.uint32)
            labels = np.arange(V, dtype=np.uint32)
            st = gg.CCStats()
            st.num_vertices = V
            st.components = c.ctypes.data_as(C.POINTER(C.c_uint32))
            st.counts = counts.ctypes.data_as(C.POINTER(C.c_uint32))
            st.labels = labels.ctypes.data_as(C.POINTER(C.c_uint32))
            lib.printCCStats(C.byref(st))
            out.append((counts, labels))
        R.ref_cc_reset()
        np.testing.assert_array_equal(out[0][0], out[1][0], err_msg=f"counts V={V}")
        np.testing.assert_array_equal(out[0][1], out[1][1], err_msg=f"labels V={V}")
    C.CDLL(None).fflush(None)
    capfd.readouterr()


def test_golden_files_reproduce_from_the_reference(orc):
    """Where the reference tree is mounted: every golden_<graph>.npz and
    fixtures.npz is exactly what tests/golden/make_golden.py computes from
    the reference's own code now (same keys, bit-identical arrays)."""
    import importlib.util

    if orc.ref_lib() is None:
        pytest.skip("reference tree not mounted here")
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    if not os.path.isdir(mg.TEST):
        pytest.skip("reference fixtures not mounted here")
    gs, fx = mg.graphs()
    z = np.load(os.path.join(GOLDEN, "fixtures.npz"))
    assert sorted(z.files) == sorted(fx)
    for k in fx:
        np.testing.assert_array_equal(z[k], fx[k], err_msg=k)
    assert sorted(gs) == sorted(NAMES)
    for name, g in gs.items():
        want = mg.golden(g)
        z = np.load(os.path.join(GOLDEN, f"golden_{name}.npz"))
        assert sorted(z.files) == sorted(want), name
        for k, v in want.items():
            a, b = np.asarray(z[k]), np.asarray(v)
            assert a.dtype == b.dtype and a.shape == b.shape, (name, k)
            assert a.tobytes() == b.tobytes(), (name, k)


def test_oracle_vs_reference_live(orc):
    """Fresh random graphs through the reference's compiled code."""
    if orc.ref_lib() is None:
        pytest.skip("reference tree not mounted here")
    rng = np.random.default_rng(11)
    for trial in range(4):
        V = int(rng.integers(20, 400))
        E = int(rng.integers(0, 6 * V))
        src = rng.integers(0, V, E).astype(np.uint32)
        dst = rng.integers(0, V, E).astype(np.uint32)
        g = orc.Csr(V, src, dst)
        for mode in range(14):
            a, ia = orc.pagerank(g, mode, 15, 1e-4)
            b, ib = orc.ref_pagerank(g, mode, 15, 1e-4)
            np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))
            assert ia["iterations"] == ib["iterations"]
        for mode in range(5):
            s = int(rng.integers(0, V))
            p, d, i1 = orc.bfs(g, mode, s)
            rp, rd, i2 = orc.ref_bfs(g, mode, s)
            np.testing.assert_array_equal(d, rd)
            np.testing.assert_array_equal(p, rp)
            assert i1["processed_nodes"] == i2["processed_nodes"] and i1["iteration"] == i2["iteration"]
        want = orc.cc_min_label(g)
        for mode in (1, 2):
            comp, _, _, info = orc.ref_cc(g, mode)
            np.testing.assert_array_equal(comp, want)
            # the reference's verify inverts its own flag: a correct
            # labelling reads FAIL (connectedComponents.c:722-832)
            assert info["verify"] == 0


def test_oracle_fp64_close_to_fp32(orc):
    g = orc.rmat_csr(12, 16)
    r32, info = orc.pagerank(g, 0, 30, 0.0)
    r64 = orc.pagerank_f64(g, info["executed"])
    assert np.abs(r32 - r64).sum() / np.abs(r64).sum() < 1e-5
    assert info["executed"] == 30


def test_oracle_planted_error_is_caught(orc):
    """A corrupted oracle input must change the compared output (the checks
    above are not vacuous)."""
    g = orc.rmat_csr(10, 16)
    r, _ = orc.pagerank(g, 2, 10, 1e-4)
    bad_adj = g.in_adj.copy()
    bad_adj[0] = (bad_adj[0] + 1) % g.V
    gb = orc.Csr.from_arrays(g.V, g.E, g.out_off, g.out_adj, g.in_off, bad_adj)
    rb, _ = orc.pagerank(gb, 2, 10, 1e-4)
    assert not np.array_equal(r, rb)


def test_oracle_ppr_seed_sets(orc):
    """Personalised PageRank from a seed set: one seed is the single-seed
    oracle, and the map from teleport vector to ranks is linear, so seeds
    {a, b} give the mean of the two single-seed vectors; repeats weigh."""
    g = orc.rmat_csr(11, 16)
    a, b = 5, 77
    ra, rb = orc.ppr_f64(g, a, 20), orc.ppr_f64(g, b, 20)
    np.testing.assert_array_equal(orc.ppr_f64_multi(g, [a], 20), ra)
    np.testing.assert_allclose(orc.ppr_f64_multi(g, [a, b], 20), 0.5 * (ra + rb), rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(orc.ppr_f64_multi(g, [a, a, b], 20), (2 * ra + rb) / 3, rtol=1e-12, atol=1e-15)
    # mass leaks only through vertices without out-edges
    assert orc.ppr_f64_multi(g, [a, b], 20).sum() <= 1.0 + 1e-12


def test_oracle_ppr_f32_batch_against_fp64(orc):
    """The batched FP32 PPR (the CPU timing baseline of the batched GPU
    form) agrees with the FP64 oracle per vector within the FP32 bar
    (L1 <= 1e-6), whatever the thread count, and an empty set stays zero."""
    g = orc.rmat_csr(12, 16)
    rng = np.random.default_rng(4)
    sets = [[int(x) for x in rng.integers(0, g.V, int(rng.integers(1, 6)))] for _ in range(20)]
    sets[3] = [sets[2][0]] * 2 + [7]
    sets[5] = []
    r = orc.ppr_f32_batch(g, sets, 20, float(np.float32(0.85)))
    r1 = orc.ppr_f32_batch(g, sets, 20, float(np.float32(0.85)), nthreads=1)
    np.testing.assert_array_equal(r, r1)   # per-vertex sums in CSC order
    for k, s in enumerate(sets):
        if not s:
            assert not r[:, k].any()
            continue
        ex = orc.ppr_f64_multi(g, s, 20, float(np.float32(0.85)))
        assert np.abs(r[:, k] - ex).sum() <= 1e-6, k


def _cc_golden():
    z = np.load(os.path.join(GOLDEN, "golden_cc.npz"))
    names = sorted({k.rsplit("_", 1)[0] for k in z.files})
    return z, names


@pytest.mark.parametrize("name", _cc_golden()[1])
def test_oracle_cc_matches_golden(orc, name):
    """Connected components: the union-find oracle, the serial
    Shiloach-Vishkin restatement and the OpenMP Afforest baseline all give
    the golden labels (smallest id of each weakly connected component, from
    scipy, tests/golden/make_cc_golden.py)."""
    z, _ = _cc_golden()
    V = int(z[name + "_V"])
    g = orc.Csr(V, z[name + "_src"], z[name + "_dst"])
    gold = z[name + "_comp"]
    np.testing.assert_array_equal(orc.cc_min_label(g), gold)
    comp, iters = orc.cc_sv(g)
    np.testing.assert_array_equal(comp, gold)
    assert iters >= 1
    np.testing.assert_array_equal(orc.cc_afforest(g, nthreads=4), gold)
    # Afforest with a sample that can only pick the largest component still
    # needs the in-edges on a directed graph; with them any sample is exact
    np.testing.assert_array_equal(orc.cc_afforest(g, samples=1, seed=5, nthreads=2), gold)


def test_oracle_cc_planted_error_is_caught(orc):
    """A labelling with one vertex moved to another component fails the
    golden comparison."""
    z, _ = _cc_golden()
    g = orc.Csr(int(z["bridged_V"]), z["bridged_src"], z["bridged_dst"])
    comp = orc.cc_min_label(g)
    comp[150] = 0
    assert not np.array_equal(comp, z["bridged_comp"])


def test_cc_golden_reproduces_from_its_script():
    """tests/golden/golden_cc.npz is what make_cc_golden.py computes (scipy)."""
    pytest.importorskip("scipy")
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_cc_golden", os.path.join(GOLDEN, "make_cc_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    z, names = _cc_golden()
    for name in names:
        V = int(z[name + "_V"])
        np.testing.assert_array_equal(mod.min_labels(V, z[name + "_src"], z[name + "_dst"]), z[name + "_comp"],
                                      err_msg=name)


def test_relabel_oracle_against_a_per_vertex_loop(orc):
    """The numpy restatement of the -l modes against a plain loop that builds
    each mode's order vertex by vertex."""
    rng = np.random.default_rng(8)
    V, E = 300, 2000
    src = rng.integers(0, V, E)
    dst = (rng.zipf(1.5, E) % V).astype(np.int64)
    dout = [0] * V
    din = [0] * V
    for a, b in zip(src, dst):
        dout[a] += 1
        din[b] += 1
    avg = E // V
    for lmode in range(10):
        deg = [dout[v] if lmode in (1, 4, 6, 8) else din[v] if lmode in (2, 5, 7, 9) else dout[v] + din[v]
               for v in range(V)]
        if lmode == 0:
            order = list(range(V))
        elif lmode in (1, 2, 3):
            order = sorted(range(V), key=lambda v: (-deg[v], v))
        elif lmode in (4, 5):
            def group(d):
                r = 2 * d // max(avg, 1)
                return min(7, r.bit_length())
            order = sorted(range(V), key=lambda v: (-group(deg[v]), v))
        elif lmode in (6, 7):
            hubs = sorted((v for v in range(V) if deg[v] > avg), key=lambda v: (-deg[v], v))
            order = hubs + [v for v in range(V) if deg[v] <= avg]
        else:
            order = [v for v in range(V) if deg[v] > avg] + [v for v in range(V) if deg[v] <= avg]
        want = np.empty(V, np.uint32)
        want[np.array(order)] = np.arange(V, dtype=np.uint32)
        np.testing.assert_array_equal(orc.relabel_order(src, dst, V, lmode), want, err_msg=f"mode {lmode}")
