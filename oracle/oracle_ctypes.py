"""ctypes bindings of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Used by tests/, ``__graft_entry__.smoke()`` (to check its results) and the CPU
baseline leg of ``bench.py``.  The product library never imports this module.

``liboracle.so`` is the plain-C restatement of the reference's CSR loops
(oracle.c).  ``_ref/libref.so`` is the reference's own pageRank.c / BFS.c /
SPMV.c compiled with stand-in headers (build_ref.sh); it exists only where the
reference tree is mounted.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = None

u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


class OrcCsr(C.Structure):
    _fields_ = [("V", C.c_uint32), ("E", C.c_uint32),
                ("out_off", C.c_void_p), ("out_adj", C.c_void_p), ("out_w", C.c_void_p),
                ("in_off", C.c_void_p), ("in_adj", C.c_void_p), ("in_w", C.c_void_p)]


class OrcPrOut(C.Structure):
    _fields_ = [("iterations", C.c_uint32), ("active", C.c_uint32), ("error_total", C.c_double),
                ("rank_sum", C.c_double), ("executed", C.c_uint32)]


class OrcBfsOut(C.Structure):
    _fields_ = [("processed_nodes", C.c_uint32), ("iteration", C.c_uint32), ("top_down_steps", C.c_uint32),
                ("bottom_up_steps", C.c_uint32), ("edges_examined", C.c_uint64),
                ("valid_source", C.c_int)]


def build():
    """Compile liboracle.so (and _ref/libref.so where the reference exists)."""
    subprocess.check_call(["make", "-s", "-C", HERE])
    subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh")])


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            subprocess.check_call(["make", "-s", "-C", HERE])
        L = C.CDLL(path)
        L.orc_rmat_edges.argtypes = [C.c_uint32, C.c_double, C.c_double, C.c_double, C.c_uint64,
                                     C.c_uint64, C.c_uint64, u32p, u32p]
        L.orc_rmat_weights.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64, f32p]
        L.orc_build_csr.argtypes = [C.c_uint32, C.c_uint32, u32p, u32p, C.c_void_p, C.c_int,
                                    u32p, u32p, C.c_void_p]
        L.orc_pagerank.argtypes = [C.POINTER(OrcCsr), C.c_int, C.c_uint32, C.c_double, C.c_int,
                                   f32p, C.POINTER(OrcPrOut), C.c_int]
        L.orc_pagerank.restype = C.c_int
        L.orc_pagerank_dd_sync.argtypes = [C.POINTER(OrcCsr), C.c_int, C.c_uint32, C.c_double, f32p]
        L.orc_pagerank_f64.argtypes = [C.POINTER(OrcCsr), C.c_uint32, C.c_int, f64p]
        L.orc_ppr_f64.argtypes = [C.POINTER(OrcCsr), C.c_uint32, C.c_uint32, C.c_double, f64p]
        L.orc_ppr_f64_multi.argtypes = [C.POINTER(OrcCsr), u32p, C.c_uint32, C.c_uint32, C.c_double, f64p]
        L.orc_ppr_f32_batch.argtypes = [C.POINTER(OrcCsr), C.c_uint32, f32p, C.c_uint32, C.c_float, C.c_int, f32p]
        L.orc_bfs.argtypes = [C.POINTER(OrcCsr), C.c_int, C.c_int, i32p, u32p, C.POINTER(OrcBfsOut), C.c_int]
        L.orc_spmv.argtypes = [C.POINTER(OrcCsr), C.c_int, C.c_uint32, C.c_void_p, f32p, f32p,
                               C.POINTER(C.c_double), C.c_int]
        L.orc_spmv.restype = C.c_int
        L.orc_spmv_f64.argtypes = [C.POINTER(OrcCsr), f32p, f64p]
        L.orc_cc_min_label.argtypes = [C.POINTER(OrcCsr), u32p]
        L.orc_cc_sv.argtypes = [C.POINTER(OrcCsr), u32p]
        L.orc_cc_sv.restype = C.c_uint32
        L.orc_cc_afforest.argtypes = [C.POINTER(OrcCsr), C.c_uint32, C.c_uint32, C.c_uint64, C.c_int, u32p,
                                      C.c_int]
        _LIB = L
    return _LIB


def ref_lib():
    """The reference's own code (None where it could not be built)."""
    global _REF
    if _REF is None:
        path = os.path.join(HERE, "_ref", "libref.so")
        if not os.path.exists(path):
            try:
                subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh")])
            except Exception:
                return None
        if not os.path.exists(path):
            return None
        R = C.CDLL(path)
        R.ref_pagerank.argtypes = [C.c_int, C.c_uint32, C.c_uint32, u32p, u32p, u32p, u32p,
                                   C.c_uint32, C.c_double, f32p, C.POINTER(C.c_uint32),
                                   C.POINTER(C.c_double)]
        R.ref_bfs.argtypes = [C.c_int, C.c_uint32, C.c_uint32, u32p, u32p, u32p, u32p, C.c_int,
                              i32p, u32p, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                              C.POINTER(C.c_int)]
        R.ref_spmv.argtypes = [C.c_int, C.c_uint32, C.c_uint32, u32p, u32p, C.c_void_p, u32p, u32p,
                               C.c_void_p, C.c_uint32, f32p, f32p]
        R.ref_cc.argtypes = [C.c_int, C.c_uint32, C.c_uint32, u32p, u32p, u32p, u32p, u32p, u32p, u32p,
                             C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), u32p, C.POINTER(C.c_uint32)]
        R.ref_set_quiet.argtypes = [C.c_int]
        _REF = R
    return _REF


# ---------------------------------------------------------------------------
# graph construction
# ---------------------------------------------------------------------------

def rmat_edges(scale, edge_factor, a=0.57, b=0.19, c=0.19, seed=27491095, weighted=False,
               weight_seed=27491095 + 2, symmetric=False):
    E = (1 << scale) * edge_factor
    src = np.empty(E, np.uint32)
    dst = np.empty(E, np.uint32)
    lib().orc_rmat_edges(scale, a, b, c, seed, 0, E, src, dst)
    w = None
    if weighted:
        w = np.empty(E, np.float32)
        lib().orc_rmat_weights(weight_seed, 0, E, w)
    if symmetric:
        src, dst = np.concatenate([src, dst]), np.concatenate([dst, src])
        if w is not None:
            w = np.concatenate([w, w])
    return src, dst, w


class Csr:
    """CSR + CSC arrays of one graph (numpy), as the oracle sees it."""

    def __init__(self, V, src, dst, w=None):
        src = np.ascontiguousarray(src, np.uint32)
        dst = np.ascontiguousarray(dst, np.uint32)
        E = len(src)
        self.V, self.E = int(V), int(E)
        self.out_off = np.empty(V + 1, np.uint32)
        self.out_adj = np.empty(max(E, 1), np.uint32)
        self.in_off = np.empty(V + 1, np.uint32)
        self.in_adj = np.empty(max(E, 1), np.uint32)
        self.out_w = self.in_w = None
        wp = None
        if w is not None:
            w = np.ascontiguousarray(w, np.float32)
            self.out_w = np.empty(max(E, 1), np.float32)
            self.in_w = np.empty(max(E, 1), np.float32)
            wp = w.ctypes.data
        L = lib()
        L.orc_build_csr(V, E, src, dst, wp, 0, self.out_off, self.out_adj,
                        None if w is None else self.out_w.ctypes.data)
        L.orc_build_csr(V, E, src, dst, wp, 1, self.in_off, self.in_adj,
                        None if w is None else self.in_w.ctypes.data)
        self._keep = (src, dst, w)

    @classmethod
    def from_arrays(cls, V, E, out_off, out_adj, in_off, in_adj, out_w=None, in_w=None):
        self = cls.__new__(cls)
        self.V, self.E = int(V), int(E)
        self.out_off = np.ascontiguousarray(out_off, np.uint32)
        self.out_adj = np.ascontiguousarray(out_adj, np.uint32)
        self.in_off = np.ascontiguousarray(in_off, np.uint32)
        self.in_adj = np.ascontiguousarray(in_adj, np.uint32)
        self.out_w = None if out_w is None else np.ascontiguousarray(out_w, np.float32)
        self.in_w = None if in_w is None else np.ascontiguousarray(in_w, np.float32)
        self._keep = ()
        return self

    def out_degree(self):
        return np.diff(self.out_off.astype(np.int64)).astype(np.uint32)

    def c(self):
        s = OrcCsr()
        s.V, s.E = self.V, self.E
        s.out_off, s.out_adj = self.out_off.ctypes.data, self.out_adj.ctypes.data
        s.in_off, s.in_adj = self.in_off.ctypes.data, self.in_adj.ctypes.data
        s.out_w = None if self.out_w is None else self.out_w.ctypes.data
        s.in_w = None if self.in_w is None else self.in_w.ctypes.data
        return s


def rmat_csr(scale, edge_factor, weighted=False, symmetric=False, seed=27491095):
    src, dst, w = rmat_edges(scale, edge_factor, seed=seed, weighted=weighted, symmetric=symmetric)
    return Csr(1 << scale, src, dst, w)


# ---------------------------------------------------------------------------
# algorithms
# ---------------------------------------------------------------------------

def pagerank(g: Csr, mode=0, iterations=20, epsilon=1e-4, init_one_over_n=False, nthreads=1):
    ranks = np.empty(g.V, np.float32)
    out = OrcPrOut()
    cs = g.c()
    rc = lib().orc_pagerank(C.byref(cs), mode, iterations, epsilon, int(init_one_over_n), ranks,
                            C.byref(out), nthreads)
    if rc != 0:
        raise ValueError(f"oracle pagerank: bad mode {mode}")
    return ranks, {"iterations": out.iterations, "active": out.active,
                   "error_total": out.error_total, "rank_sum": out.rank_sum,
                   "executed": out.executed}


def pagerank_dd_sync(g: Csr, mode, iterations=20, epsilon=1e-4):
    """Data-driven push (7) / pull-push (8) in the synchronous order."""
    ranks = np.empty(g.V, np.float32)
    cs = g.c()
    lib().orc_pagerank_dd_sync(C.byref(cs), mode, iterations, epsilon, ranks)
    return ranks


def pagerank_f64(g: Csr, executed, init_one_over_n=False):
    r = np.empty(g.V, np.float64)
    cs = g.c()
    lib().orc_pagerank_f64(C.byref(cs), executed, int(init_one_over_n), r)
    return r


def ppr_f64(g: Csr, seed_vertex, iterations, damp=0.85):
    r = np.empty(g.V, np.float64)
    cs = g.c()
    lib().orc_ppr_f64(C.byref(cs), seed_vertex, iterations, damp, r)
    return r


def ppr_f64_multi(g: Csr, seeds, iterations, damp=0.85):
    """FP64 personalised PageRank from a seed set (repeats allowed)."""
    s = np.ascontiguousarray(seeds, np.uint32)
    r = np.empty(g.V, np.float64)
    cs = g.c()
    lib().orc_ppr_f64_multi(C.byref(cs), s, len(s), iterations, damp, r)
    return r


def ppr_f32_batch(g: Csr, sets, iterations, damp=0.85, nthreads=0):
    """K seed sets advanced together in FP32 on the host cores ([V][K])."""
    K = len(sets)
    share = np.zeros((g.V, K), np.float64)
    for k, s in enumerate(sets):
        for v in s:
            share[v, k] += 1.0 / len(s)
    init = share.astype(np.float32)
    r = np.empty((g.V, K), np.float32)
    cs = g.c()
    lib().orc_ppr_f32_batch(C.byref(cs), K, init, iterations, damp, nthreads, r)
    return r


def bfs(g: Csr, mode=2, source=0, nthreads=1):
    parents = np.empty(g.V, np.int32)
    dist = np.empty(g.V, np.uint32)
    out = OrcBfsOut()
    cs = g.c()
    lib().orc_bfs(C.byref(cs), mode, source, parents, dist, C.byref(out), nthreads)
    return parents, dist, {"processed_nodes": out.processed_nodes, "iteration": out.iteration,
                           "top_down_steps": out.top_down_steps,
                           "bottom_up_steps": out.bottom_up_steps,
                           "edges_examined": out.edges_examined,
                           "valid_source": out.valid_source}


def spmv(g: Csr, mode=0, iterations=1, x=None, nthreads=1):
    xo = np.empty(g.V, np.float32)
    y = np.empty(g.V, np.float32)
    chk = C.c_double()
    xp = None
    if x is not None:
        x = np.ascontiguousarray(x, np.float32)
        xp = x.ctypes.data
    cs = g.c()
    rc = lib().orc_spmv(C.byref(cs), mode, iterations, xp, xo, y, C.byref(chk), nthreads)
    if rc != 0:
        raise ValueError(f"oracle spmv: bad mode {mode}")
    return xo, y, chk.value


def spmv_f64(g: Csr, x):
    y = np.empty(g.V, np.float64)
    cs = g.c()
    lib().orc_spmv_f64(C.byref(cs), np.ascontiguousarray(x, np.float32), y)
    return y


def cc_min_label(g: Csr):
    """Smallest vertex id of each vertex's weakly connected component."""
    comp = np.empty(g.V, np.uint32)
    cs = g.c()
    lib().orc_cc_min_label(C.byref(cs), comp)
    return comp


def cc_sv(g: Csr):
    """The reference's Shiloach-Vishkin loop, serial: (labels, iterations)."""
    comp = np.empty(g.V, np.uint32)
    cs = g.c()
    it = lib().orc_cc_sv(C.byref(cs), comp)
    return comp, int(it)


def cc_afforest(g: Csr, rounds=2, samples=1024, seed=27491095, use_in=True, nthreads=1):
    """The reference's CPU Afforest with OpenMP (the timed CPU baseline)."""
    comp = np.empty(g.V, np.uint32)
    cs = g.c()
    lib().orc_cc_afforest(C.byref(cs), rounds, samples, seed, int(use_in), comp, nthreads)
    return comp


def _splitmix64(z):
    z = z.astype(np.uint64)
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def relabel_order(src, dst, V, lmode, seed=27491095):
    """label[orig] = new for the reference's -l modes 0..10, restated from the
    published algorithms (degree sorts, DBG, HUBSort, HUBCluster, random) as
    the product documents them: one key per vertex, ties in id order."""
    src = np.asarray(src, np.int64)
    dst = np.asarray(dst, np.int64)
    E = len(src)
    dout = np.bincount(src, minlength=V).astype(np.int64)
    din = np.bincount(dst, minlength=V).astype(np.int64)
    d = {1: dout, 4: dout, 6: dout, 8: dout, 2: din, 5: din, 7: din, 9: din, 3: dout + din}.get(lmode)
    avg = E // V if V else 0
    if lmode == 0:
        key = np.zeros(V, np.int64)
    elif lmode in (1, 2, 3):
        key = d.max(initial=0) - d
    elif lmode in (4, 5):
        r = 2 * d // max(avg, 1)
        group = np.minimum(7, np.array([int(x).bit_length() for x in r], np.int64))
        key = 7 - group
    elif lmode in (6, 7):
        dmax = d.max(initial=0)
        key = np.where(d > avg, dmax - d, dmax + 1)
    elif lmode in (8, 9):
        key = np.where(d > avg, 0, 1)
    elif lmode == 10:
        key = (_splitmix64(np.uint64(seed) ^ np.arange(V, dtype=np.uint64)) & np.uint64(0xFFFFFFFF)).astype(np.int64)
    else:
        raise ValueError(f"relabel mode {lmode}")
    order = np.argsort(key, kind="stable")
    label = np.empty(V, np.uint32)
    label[order] = np.arange(V, dtype=np.uint32)
    return label


# ---------------------------------------------------------------------------
# the reference's own code (where it was built)
# ---------------------------------------------------------------------------

def ref_pagerank(g: Csr, mode=0, iterations=20, epsilon=1e-4):
    R = ref_lib()
    ranks = np.empty(g.V, np.float32)
    it = C.c_uint32()
    err = C.c_double()
    R.ref_pagerank(mode, g.V, g.E, g.out_off, g.out_adj, g.in_off, g.in_adj, iterations, epsilon,
                   ranks, C.byref(it), C.byref(err))
    return ranks, {"iterations": it.value, "error_total": err.value}


def ref_bfs(g: Csr, mode=2, source=0):
    R = ref_lib()
    parents = np.empty(g.V, np.int32)
    dist = np.empty(g.V, np.uint32)
    processed = C.c_uint32()
    iteration = C.c_uint32()
    src_out = C.c_int()
    R.ref_bfs(mode, g.V, g.E, g.out_off, g.out_adj, g.in_off, g.in_adj, source, parents, dist,
              C.byref(processed), C.byref(iteration), C.byref(src_out))
    return parents, dist, {"processed_nodes": processed.value, "iteration": iteration.value,
                           "source_out": src_out.value}


def ref_spmv(g: Csr, mode=0, iterations=1):
    R = ref_lib()
    x = np.empty(g.V, np.float32)
    y = np.empty(g.V, np.float32)
    R.ref_spmv(mode, g.V, g.E, g.out_off, g.out_adj,
               None if g.out_w is None else g.out_w.ctypes.data, g.in_off, g.in_adj,
               None if g.in_w is None else g.in_w.ctypes.data, iterations, x, y)
    return x, y


def ref_cc(g: Csr, mode=1):
    """The reference's connectedComponentsGraphCSR (1 Afforest, 2 weakly):
    components, counts, labels, {iterations, neighbor_rounds, mt: the
    generator state after the call (624 words, then the index), verify: what
    the reference's connectedComponentsVerifyGraphCSR returns for it}."""
    R = ref_lib()
    comp = np.empty(g.V, np.uint32)
    counts = np.empty(g.V, np.uint32)
    labels = np.empty(g.V, np.uint32)
    it = C.c_uint32()
    nr = C.c_uint32()
    mt = np.empty(625, np.uint32)
    ver = C.c_uint32()
    rc = R.ref_cc(mode, g.V, g.E, g.out_off, g.out_adj, g.in_off, g.in_adj, comp, counts, labels,
                  C.byref(it), C.byref(nr), mt, C.byref(ver))
    if rc != 0:
        raise ValueError(f"ref_cc mode {mode}")
    return comp, counts, labels, {"iterations": it.value, "neighbor_rounds": nr.value, "mt": mt,
                                  "verify": ver.value}


# ---------------------------------------------------------------------------
# BFS checks shared by the tests
# ---------------------------------------------------------------------------

def bfs_levels_reference(g: Csr, source):
    """Exact BFS levels over out-edges (-1 = unreached), by a plain queue."""
    lev = np.full(g.V, -1, np.int64)
    if source >= g.V:
        return lev
    lev[source] = 0
    frontier = np.array([source], np.int64)
    d = 0
    off, adj = g.out_off.astype(np.int64), g.out_adj
    while len(frontier):
        d += 1
        starts, ends = off[frontier], off[frontier + 1]
        nb = np.concatenate([adj[s:e] for s, e in zip(starts, ends)]) if len(frontier) else np.array([])
        nb = np.unique(nb.astype(np.int64))
        nb = nb[lev[nb] < 0]
        lev[nb] = d
        frontier = nb
    return lev


def check_parents(g: Csr, source, parents, levels):
    """Every reached vertex other than the source has a parent one level up
    with an edge parent -> vertex; unreached vertices keep a negative parent."""
    V = g.V
    reached = levels >= 0
    if source < V:
        assert parents[source] == source
    bad = []
    off = g.out_off.astype(np.int64)
    for v in np.nonzero(reached)[0]:
        if v == source:
            continue
        p = int(parents[v])
        if p < 0 or p >= V or levels[p] != levels[v] - 1:
            bad.append(v)
            continue
        nbrs = g.out_adj[off[p]:off[p + 1]]
        if not np.any(nbrs == v):
            bad.append(v)
    assert not bad, f"{len(bad)} vertices with invalid parents, first {bad[:5]}"
    assert np.all(parents[~reached] < 0)
