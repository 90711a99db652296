"""Host-side pieces of the product on CPU: the C-ABI library loads and
exports every function include/*.h declares; the graph builder, R-MAT
generator and edge-list loaders agree with the oracle's independent ones;
host utilities behave like the reference's OpenGraph helpers.  No GPU
compute is called."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from graphs import fixture_edges

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b([A-Za-z_]\w*)\s*\(([^;{]*)\)\s*;", text, flags=re.M):
            if m.group(0).lstrip().startswith(("typedef", "#", "return")):
                continue
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_function(gg):
    names = _declared_functions()
    assert len(names) > 80
    L = gg.lib()
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing


def _reference_root():
    """The reference snapshot's root, as tests/golden/make_golden.py names
    it, or None where it is not mounted."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_golden",
                                                  os.path.join(ROOT, "tests", "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg.REF if os.path.isdir(os.path.join(mg.REF, "02_capi_graph")) else None


def test_reference_headers_csr_entry_points_are_exported(gg):
    """Where the reference tree is mounted: every function its four
    algorithm headers declare is exported by the library, except the members
    for other graph layouts (Grid, AdjArrayList, AdjLinkedList), the BFS
    DualOrder variants and their helpers, the Judy sampling helper addSample
    (sampling runs on the device), bottomUpStepGraphCSRCAPI (its arguments
    are the FPGA's status and handle, the layer the GPU runtime replaces)
    and pageRankCompare (declared by the reference, defined nowhere in
    it)."""
    ref = _reference_root()
    if ref is None:
        pytest.skip("reference tree not mounted here")
    hdrs = os.path.join(ref, "02_capi_graph", "include", "algorithms", "capi")
    other_layout = re.compile(r"Grid|AdjArrayList|AdjLinkedList|DualOrder")
    decl = re.compile(r"^[A-Za-z_][\w \*]*?[ \*](\w+)\s*\(")
    want = set()
    for h in ("pageRank.h", "BFS.h", "SPMV.h", "connectedComponents.h"):
        for line in open(os.path.join(hdrs, h)):
            m = decl.match(line)
            if m and not other_layout.search(line) and m.group(1) not in ("addSample", "bottomUpStepGraphCSRCAPI",
                                                                              "pageRankCompare"):
                want.add(m.group(1))
    assert len(want) > 40, sorted(want)
    L = gg.lib()
    missing = [n for n in sorted(want) if not hasattr(L, n)]
    assert not missing, missing


def test_struct_layouts_match_the_reference_headers(gg, tmp_path):
    """Where the reference tree is mounted: struct Arguments and the four
    stats structs have the reference's size and every field's offset (one
    probe compiled against the reference's headers, with the oracle's
    stand-ins for its absent OpenGraph headers, and against include/)."""
    import subprocess

    ref = _reference_root()
    if ref is None:
        pytest.skip("reference tree not mounted here")
    structs = {"Arguments": gg.Arguments, "PageRankStats": gg.PageRankStats, "BFSStats": gg.BFSStats,
               "SPMVStats": gg.SPMVStats, "CCStats": gg.CCStats}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "graphConfig.h"', '#include "pageRank.h"',
             '#include "BFS.h"', '#include "SPMV.h"', '#include "connectedComponents.h"', "int main(void)", "{"]
    for name, cls in structs.items():
        lines.append(f'    printf("{name} %zu\\n", sizeof(struct {name}));')
        for field, _ in cls._fields_:
            lines.append(f'    printf("{name}.{field} %zu\\n", offsetof(struct {name}, {field}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")

    def run(incs, tag):
        exe = tmp_path / f"layout_{tag}"
        subprocess.check_call(["gcc", "-std=gnu11", "-w", *incs, str(src), "-o", str(exe)])
        return subprocess.check_output([str(exe)], text=True)

    inc = os.path.join(ref, "02_capi_graph", "include")
    theirs = run(["-I" + os.path.join(ROOT, "oracle", "ref_shim"), "-I" + os.path.join(inc, "config"),
                  "-I" + os.path.join(inc, "algorithms", "capi"), "-I" + os.path.join(inc, "capi_utils")], "ref")
    ours = run(["-I" + os.path.join(ROOT, "include")], "ours")
    assert len(theirs.splitlines()) > 60
    assert ours == theirs


def test_struct_sizes_match_c_layout(gg, tmp_path):
    """The ctypes mirror has the C compiler's layout of every drop-in struct."""
    structs = {"Arguments": gg.Arguments, "GraphCSR": gg.GraphCSR, "EdgeList": gg.EdgeList,
               "Vertex": gg.Vertex, "PageRankStats": gg.PageRankStats, "BFSStats": gg.BFSStats,
               "SPMVStats": gg.SPMVStats, "Bitmap": gg.Bitmap, "ArrayQueue": gg.ArrayQueue,
               "CCStats": gg.CCStats}
    typedefs = {"gg_pr_params": gg.PrParams, "gg_pr_result": gg.PrResult, "gg_bfs_params": gg.BfsParams,
                "gg_bfs_result": gg.BfsResult, "gg_spmv_params": gg.SpmvParams, "gg_spmv_result": gg.SpmvResult,
                "GraphGpuOptions": gg.GraphGpuOptions, "gg_ppr_params": gg.PprParams, "gg_ppr_result": gg.PprResult,
                "gg_cc_params": gg.CcParams, "gg_cc_result": gg.CcResult}
    src = ['#include <stdio.h>', '#include "pageRank.h"', '#include "BFS.h"', '#include "SPMV.h"',
           '#include "connectedComponents.h"', '#include "gg_runtime.h"', "int main(void){"]
    for n in structs:
        src.append(f'printf("{n} %zu\\n", sizeof(struct {n}));')
    for n in typedefs:
        src.append(f'printf("{n} %zu\\n", sizeof({n}));')
    src.append("return 0;}")
    (tmp_path / "sz.c").write_text("\n".join(src))
    import subprocess
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(tmp_path / "sz.c"), "-o",
                           str(tmp_path / "sz")])
    out = subprocess.check_output([str(tmp_path / "sz")]).decode().split("\n")
    sizes = dict(line.split() for line in out if line)
    for n, t in {**structs, **typedefs}.items():
        assert int(sizes[n]) == C.sizeof(t), n
    a = gg.default_arguments()
    assert a.iterations == 20 and abs(a.epsilon - 1e-4) < 1e-15 and a.binSize == 512
    assert a.mt19937var.mt[0] == 27491095 and a.cu_config == 1


def test_mt19937_known_answer(gg):
    # first outputs of MT19937 seeded with 5489 (the generator's published test value)
    st = gg.Mt19937State()
    gg.lib().initializeMersenneState(C.byref(st), 5489)
    gg.lib().generateRandInt.restype = C.c_uint32
    outs = [gg.lib().generateRandInt(C.byref(st)) for _ in range(3)]
    assert outs == [3499211612, 581869302, 3890346734]


@pytest.mark.parametrize("scale,ef,weighted,sym", [(6, 4, False, False), (10, 16, True, False), (12, 8, True, True)])
def test_builder_matches_oracle(gg, orc, scale, ef, weighted, sym):
    g = gg.Graph.rmat(scale, ef, weighted=weighted, symmetric=sym)
    a = g.arrays()
    src, dst, w = orc.rmat_edges(scale, ef, weighted=weighted, symmetric=sym)
    o = orc.Csr(1 << scale, src, dst, w)
    for k in ["out_off", "out_adj", "in_off", "in_adj"]:
        np.testing.assert_array_equal(a[k], getattr(o, k), err_msg=k)
    np.testing.assert_array_equal(a["out_degree"], np.diff(o.out_off))
    np.testing.assert_array_equal(a["in_degree"], np.diff(o.in_off))
    if weighted:
        np.testing.assert_array_equal(a["out_w"], o.out_w)
        np.testing.assert_array_equal(a["in_w"], o.in_w)
    assert g.E == len(src) and g.V == 1 << scale


def test_rmat_statistics(orc):
    """Quadrant frequencies follow (a, b, c, d) = (0.57, 0.19, 0.19, 0.05) at the top level."""
    src, dst, _ = orc.rmat_edges(14, 16)
    top_s, top_d = src >> 13, dst >> 13
    q = np.bincount(top_s * 2 + top_d, minlength=4) / len(src)
    np.testing.assert_allclose(q, [0.57, 0.19, 0.19, 0.05], atol=0.005)


def test_builder_on_reference_fixtures(gg, orc):
    for name, (s, d, w) in fixture_edges().items():
        g = gg.Graph.from_edges(s, d, w)
        a = g.arrays()
        o = orc.Csr(g.V, s, d, w)
        np.testing.assert_array_equal(a["in_adj"][:g.E], o.in_adj[:g.E])
        np.testing.assert_array_equal(a["out_off"], o.out_off)


def test_loaders_read_reference_formats(gg, tmp_path):
    src = np.array([1, 2, 3, 0], np.uint32)
    dst = np.array([2, 3, 0, 1], np.uint32)
    np.stack([src, dst], 1).astype(np.uint32).tofile(tmp_path / "g.bin")
    np.stack([src, dst, np.array([5, 6, 7, 8])], 1).astype(np.uint32).tofile(tmp_path / "g.wbin")
    (tmp_path / "g.txt").write_text("1 2\n2 3\n3 0\n0 1\n")
    for f, w in [("g.bin", False), ("g.wbin", True), ("g.txt", False)]:
        g = gg.Graph.from_file(str(tmp_path / f), weighted=w)
        a = g.arrays()
        assert g.V == 4 and g.E == 4
        np.testing.assert_array_equal(a["out_adj"], [1, 2, 3, 0])
        if w:
            np.testing.assert_array_equal(a["out_w"], [8, 5, 6, 7])
    assert not gg.lib().readEdgeListsbin(str(tmp_path / "missing.bin").encode(), 0)


def test_empty_and_tiny_graphs(gg):
    g = gg.Graph.from_edges(np.zeros(0, np.uint32), np.zeros(0, np.uint32), num_vertices=3)
    a = g.arrays()
    assert g.E == 0 and list(a["out_off"]) == [0, 0, 0, 0]
    g = gg.Graph.from_edges([0, 0, 0], [0, 0, 1])  # self loops and duplicates kept
    a = g.arrays()
    assert list(a["out_adj"]) == [0, 0, 1] and list(a["in_off"]) == [0, 2, 3]


def test_bitmap_and_queue_helpers(gg):
    L = gg.lib()
    b = L.newBitmap(100)
    for v in (0, 31, 32, 99):
        L.setBit(b, v)
    assert L.getNumOfSetBits(b) == 4
    L.freeBitmap(b)
    q = L.newArrayQueue(10)
    L.enArrayQueue(q, 4)
    L.enArrayQueue(q, 7)
    assert q.contents.tail - q.contents.head == 2
    L.freeArrayQueue(q)


def test_gpu_calls_fail_loudly_without_device(gg):
    """On a machine without a GPU the runtime reports an error instead of
    computing on the CPU."""
    n = C.c_int(0)
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    st = gg.lib().gg_device_init(0)
    assert st != 0
    g = gg.Graph.rmat(6, 4)
    assert not gg.lib().pageRankGraphCSR(C.byref(gg.default_arguments()), g.ptr)
    assert gg.lib().graphGpuLastError() != 0


def test_host_copy_mode_and_device_cache_controls(gg):
    """The copy-route setting round-trips, an unknown route falls back to
    auto, and the device-block cache controls work before any device
    memory was allocated (an empty cache, nothing to trim)."""
    L = gg.lib()
    before = L.gg_host_copy_mode()
    try:
        for name, value in gg.HOST_COPY.items():
            gg.set_host_copy_mode(name)
            assert L.gg_host_copy_mode() == value, name
        L.gg_set_host_copy_mode(99)
        assert L.gg_host_copy_mode() == gg.HOST_COPY["auto"]
    finally:
        L.gg_set_host_copy_mode(before)
    gg.device_cache_trim()
    assert gg.device_cache_bytes() == 0


def test_rmat_batch_is_union_of_single_graphs(gg):
    """generateRMATBatchEdgeList: block i of the union is exactly the R-MAT
    graph of scale scales[i] and seed seed0 + i, renumbered from vertex_off[i]."""
    scales = [4, 6, 3, 7, 5]
    g, voff = gg.Graph.rmat_batch(scales, edge_factor=8, seed0=1234)
    assert list(voff) == list(np.cumsum([0] + [1 << s for s in scales]))
    a = g.arrays()
    for i, sc in enumerate(scales):
        one = gg.Graph.rmat(sc, 8, seed=1234 + i).arrays()
        lo, hi = int(voff[i]), int(voff[i + 1])
        for side in ("out", "in"):
            off, adj = a[side + "_off"], a[side + "_adj"]
            blk = off[lo:hi + 1] - off[lo]
            np.testing.assert_array_equal(blk, one[side + "_off"])
            np.testing.assert_array_equal(adj[off[lo]:off[hi]] - lo, one[side + "_adj"])


def test_cc_host_helpers_and_verify(gg, orc):
    """The drop-in's host-side connected-components pieces, without a GPU:
    linkNodes + compressNodes give the smallest-id labels; the verify
    function accepts them and rejects identity labels and a planted error."""
    import ctypes as C

    rng = np.random.default_rng(4)
    V = 500
    s = rng.integers(0, V, 600).astype(np.uint32)
    d = rng.integers(0, V, 600).astype(np.uint32)
    g = gg.Graph.from_edges(s, d, num_vertices=V)
    a = g.arrays()
    gold = orc.cc_min_label(orc.Csr.from_arrays(V, g.E, a["out_off"], a["out_adj"], a["in_off"], a["in_adj"]))
    L = gg.lib()
    comp = np.arange(V, dtype=np.uint32)
    for u, v in zip(s, d):
        L.linkNodes(int(u), int(v), comp.ctypes.data)
    L.compressNodes(V, comp.ctypes.data)
    np.testing.assert_array_equal(comp, gold)
    st = L.newCCStatsGraphCSR(g.ptr)
    try:
        assert L.connectedComponentsVerifyGraphCSR(st, g.ptr) == 0  # identity labels
        C.memmove(st.contents.components, gold.ctypes.data, V * 4)
        assert L.connectedComponentsVerifyGraphCSR(st, g.ptr) == 1
        bad = gold.copy()
        bad[np.flatnonzero(gold != np.arange(V))[0]] = V - 1 if gold[-1] != V - 1 else 0
        C.memmove(st.contents.components, bad.ctypes.data, V * 4)
        assert L.connectedComponentsVerifyGraphCSR(st, g.ptr) == 0
    finally:
        L.freeCCStats(st)


def test_cc_stats_arrays_as_the_reference_leaves_them(gg, orc, capfd):
    """printCCStats (the reference fills counts and labels there): sizes
    sorted ascending with the label of each beside it, ties by ascending id,
    the largest component last; a second call gives the same arrays; the
    table lists the largest component first."""
    import ctypes as C

    rng = np.random.default_rng(9)
    V = 700
    s = rng.integers(0, V, 500).astype(np.uint32)
    d = rng.integers(0, V, 500).astype(np.uint32)
    g = gg.Graph.from_edges(s, d, num_vertices=V)
    a = g.arrays()
    gold = orc.cc_min_label(orc.Csr.from_arrays(V, g.E, a["out_off"], a["out_adj"], a["in_off"], a["in_adj"]))
    size = np.bincount(gold, minlength=V).astype(np.uint32)
    order = np.argsort(size, kind="stable").astype(np.uint32)
    L = gg.lib()
    st = L.newCCStatsGraphCSR(g.ptr)
    try:
        C.memmove(st.contents.components, gold.ctypes.data, V * 4)
        for _ in range(2):
            L.printCCStats(st)
            counts = np.ctypeslib.as_array(st.contents.counts, (V,)).copy()
            labels = np.ctypeslib.as_array(st.contents.labels, (V,)).copy()
            np.testing.assert_array_equal(labels, order)
            np.testing.assert_array_equal(counts, size[order])
        C.CDLL(None).fflush(None)  # the table went through C stdio
        out = capfd.readouterr().out
        assert f"| {int(order[-1]):<21} | {int(size.max()):<27} |" in out
        assert f"| {'Num Components':<21} | {int((size > 0).sum()):<27} |" in out
    finally:
        L.freeCCStats(st)


def test_generator_state_as_the_reference_leaves_it(gg):
    """The drop-in's MT19937 from the reference CLI's seed, advanced by the
    reference Afforest's 1024 samples, is the generator state the
    reference's own connectedComponents.c left (golden, R-MAT-10); its
    weakly variant draws nothing."""
    import ctypes as C
    import os

    from graphs import GOLDEN

    z = np.load(os.path.join(GOLDEN, "golden_rmat10.npz"))
    a = gg.default_arguments()
    for _ in range(1024):
        gg.lib().generateRandInt(C.byref(a.mt19937var))
    np.testing.assert_array_equal(np.frombuffer(bytes(a.mt19937var), np.uint32), z["cc1_mt"])
    b = gg.default_arguments()
    np.testing.assert_array_equal(np.frombuffer(bytes(b.mt19937var), np.uint32), z["cc2_mt"])


def test_text_loader_skips_comments_and_defaults_weights(gg, tmp_path):
    """Text edge lists: comment and header lines are skipped, a missing
    weight column reads as 1, and more edges than the first buffer holds
    (1024) are kept in order."""
    lines = ["# a comment", "% a header", ""]
    rng = np.random.default_rng(1)
    src = rng.integers(0, 500, 3000)
    dst = rng.integers(0, 500, 3000)
    for k, (a, b) in enumerate(zip(src, dst)):
        lines.append(f"{a} {b} {k % 7 + 1}" if k % 2 else f"{a} {b}")
    (tmp_path / "g.txt").write_text("\n".join(lines) + "\n")
    L = gg.lib()
    el = L.readEdgeListsText(str(tmp_path / "g.txt").encode(), 1)
    assert el
    try:
        e = el.contents
        assert e.num_edges == 3000 and e.num_vertices == int(max(src.max(), dst.max())) + 1
        got_s = np.ctypeslib.as_array(e.edges_array_src, (3000,))
        got_w = np.ctypeslib.as_array(e.edges_array_weight, (3000,))
        np.testing.assert_array_equal(got_s, src.astype(np.uint32))
        want_w = np.array([(k % 7 + 1) if k % 2 else 1 for k in range(3000)], np.float32)
        np.testing.assert_array_equal(got_w, want_w)
    finally:
        L.freeEdgeList(el)


def test_binary_loader_rejects_truncated_files(gg, tmp_path):
    np.arange(7, dtype=np.uint32).tofile(tmp_path / "odd.bin")  # 28 bytes: not whole (src, dst) pairs
    assert not gg.lib().readEdgeListsbin(str(tmp_path / "odd.bin").encode(), 0)
    np.arange(8, dtype=np.uint32).tofile(tmp_path / "odd.wbin")  # 32 bytes: not whole triples
    assert not gg.lib().readEdgeListsbin(str(tmp_path / "odd.wbin").encode(), 1)


def test_every_header_compiles_alone_as_c(tmp_path):
    """Each public header is self-contained C (a reference-side caller can
    include any one of them first), with no warnings."""
    import subprocess

    inc = os.path.join(ROOT, "include")
    for h in sorted(os.listdir(inc)):
        if not h.endswith(".h"):
            continue
        src = tmp_path / "inc.c"
        src.write_text(f'#include "{h}"\nint main(void) {{ return 0; }}\n')
        r = subprocess.run(["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-I", inc, "-c", str(src), "-o",
                            str(tmp_path / "inc.o")], capture_output=True, text=True)
        assert r.returncode == 0, (h, r.stderr)
