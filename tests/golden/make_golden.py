"""Generate the golden vectors under tests/golden/ from the reference itself.

Run where the reference snapshot is available: $ACCELGRAPH_REFERENCE, or a
checkout beside this repository (../reference):

    python tests/golden/make_golden.py            # everything
    python tests/golden/make_golden.py ring hubs  # only the golden files of those graphs

It writes
  fixtures.npz  the reference's fixture graphs (04_test_graphs/TEST/*), as
                uint32 edge arrays (weights from the .wbin files), and
  golden_*.npz  outputs of the reference's own pageRank.c / BFS.c / SPMV.c /
                connectedComponents.c (Afforest and weakly; Judy arrays
                from the stand-in oracle/ref_shim/Judy.h),
                compiled from the reference sources by oracle/build_ref.sh
                (FPGA-offloaded loops replaced by the compute-unit emulation
                in oracle/ref_shim/ref_capi_emu.c), on those fixtures, on
                small seeded R-MAT graphs and on the edge-case graphs of
                tests/graphs.py (special_edges), run with one OpenMP thread.
The GPU machine has no reference tree; the tests read these files there.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle_ctypes as O  # noqa: E402

sys.path.insert(0, os.path.dirname(HERE))
from graphs import special_edges  # noqa: E402

REF = os.environ.get("ACCELGRAPH_REFERENCE", os.path.join(os.path.dirname(ROOT), "reference"))
TEST = os.path.join(REF, "04_test_graphs", "TEST")

FIXTURES = {
    "graphbrew": ("graphbrew/graph.bin", False),
    "test": ("test/graph.wbin", True),
    "v51_e1021": ("v51_e1021/graph.wbin", True),
    "v300_e2730": ("v300_e2730/graph.wbin", True),
}
RMAT = {"rmat8": (8, 8), "rmat10": (10, 16), "rmat12u": (12, 8)}
PR_ITERS, PR_EPS = 20, 1e-4
SPMV_ITERS = 3


def load(rel, weighted):
    a = np.fromfile(os.path.join(TEST, rel), dtype=np.uint32)
    k = 3 if weighted else 2
    a = a.reshape(-1, k)
    w = a[:, 2].astype(np.float32) if weighted else None
    return a[:, 0].copy(), a[:, 1].copy(), w


def sources(V):
    return sorted({0, 1, V // 2, V - 1})


def graphs():
    """(graphs by name, the fixture edge arrays for fixtures.npz)."""
    fx = {}
    out = {}
    for name, (rel, weighted) in FIXTURES.items():
        s, d, w = load(rel, weighted)
        fx[name + "_src"], fx[name + "_dst"] = s, d
        if w is not None:
            fx[name + "_w"] = w
        V = int(max(s.max(), d.max())) + 1
        out[name] = O.Csr(V, s, d, w)
    for name, (scale, ef) in RMAT.items():
        out[name] = O.rmat_csr(scale, ef, weighted=True, symmetric=name.endswith("u"))
    for name, (s, d, w, V) in special_edges().items():
        out[name] = O.Csr(V, s, d, w)
    return out, fx


def golden(g):
    """The contents of one golden_<graph>.npz: the reference's own outputs on g."""
    out = {"V": np.uint32(g.V), "E": np.uint32(g.E)}
    for mode in range(14):
        r, info = O.ref_pagerank(g, mode, PR_ITERS, PR_EPS)
        out[f"pr{mode}_ranks"] = r
        out[f"pr{mode}_iters"] = np.uint32(info["iterations"])
        out[f"pr{mode}_err"] = np.float64(info["error_total"])
    srcs = sources(g.V)
    out["bfs_sources"] = np.array(srcs, np.int32)
    for mode in range(5):
        for s in srcs:
            p, d, info = O.ref_bfs(g, mode, s)
            out[f"bfs{mode}_{s}_parents"] = p
            out[f"bfs{mode}_{s}_dist"] = d
            out[f"bfs{mode}_{s}_processed"] = np.uint32(info["processed_nodes"])
            out[f"bfs{mode}_{s}_iteration"] = np.uint32(info["iteration"])
    # the reference is built WEIGHTED 0 (graphConfig.h:7): its SpMV uses
    # the constant weight 0.0001f, so its golden runs on the unweighted view
    gu = O.Csr.from_arrays(g.V, g.E, g.out_off, g.out_adj, g.in_off, g.in_adj)
    for mode in range(4):
        x, y = O.ref_spmv(gu, mode, SPMV_ITERS)
        out[f"spmv{mode}_x"] = x
        out[f"spmv{mode}_y"] = y
    # connectedComponents.c through connectedComponentsGraphCSR: 1
    # Afforest, 2 weakly (its Shiloach-Vishkin runs on the FPGA)
    for mode in (1, 2):
        comp, counts, labels, info = O.ref_cc(g, mode)
        out[f"cc{mode}_components"] = comp
        out[f"cc{mode}_counts"] = counts
        out[f"cc{mode}_labels"] = labels
        out[f"cc{mode}_iterations"] = np.uint32(info["iterations"])
        out[f"cc{mode}_mt"] = info["mt"]
    return out


def main(only):
    if O.ref_lib() is None:
        sys.exit("the reference could not be built (is the reference tree mounted?)")
    gs, fx = graphs()
    if not only:
        np.savez_compressed(os.path.join(HERE, "fixtures.npz"), **fx)
    for name, g in gs.items():
        if only and name not in only:
            continue
        np.savez_compressed(os.path.join(HERE, f"golden_{name}.npz"), **golden(g))
        print("wrote", name, g.V, g.E)


if __name__ == "__main__":
    main(set(sys.argv[1:]))
