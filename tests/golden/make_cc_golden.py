"""Golden connected-component labels for tests/golden/golden_cc.npz.

The labels come from an independent implementation (the reference's own
Afforest and weakly variants give a second set, in golden_<graph>.npz from
make_golden.py; its Shiloach-Vishkin runs on the FPGA and is not emulated):
scipy.sparse.csgraph.connected_components with connection="weak", turned
into the labelling every reference algorithm converges to -- the smallest
vertex id of each weakly connected component.

    python tests/golden/make_cc_golden.py

Graphs: the reference's fixture graphs (fixtures.npz), seeded R-MAT graphs
(directed and symmetrised, with the oracle's generator), and edge cases
(isolated vertices, a long chain, a directed star, two cliques bridged by
one directed edge).  Edges are stored beside the labels.
"""
import os
import sys

import numpy as np
import scipy.sparse as sp
from scipy.sparse.csgraph import connected_components

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle_ctypes as O  # noqa: E402


def min_labels(V, src, dst):
    A = sp.coo_matrix((np.ones(len(src), np.int8), (src.astype(np.int64), dst.astype(np.int64))), shape=(V, V))
    n, lab = connected_components(A, directed=True, connection="weak")
    mins = np.full(n, V, np.int64)
    np.minimum.at(mins, lab, np.arange(V))
    return mins[lab].astype(np.uint32)


def graphs():
    out = {}
    z = np.load(os.path.join(HERE, "fixtures.npz"))
    for name in ["graphbrew", "test", "v51_e1021", "v300_e2730"]:
        s, d = z[name + "_src"], z[name + "_dst"]
        out[name] = (int(max(s.max(), d.max())) + 1, s, d)
    for name, (scale, ef, sym) in {"rmat10": (10, 2, False), "rmat12u": (12, 1, True),
                                   "rmat14": (14, 4, False)}.items():
        s, d, _ = O.rmat_edges(scale, ef, symmetric=sym)
        out[name] = (1 << scale, s, d)
    rng = np.random.default_rng(11)
    chain = np.arange(0, 3000, dtype=np.uint32)
    out["chain_rev"] = (3001, chain[::-1] + 1, chain[::-1])          # 3000 -> 2999 -> ... -> 0
    star = np.arange(1, 2001, dtype=np.uint32)
    out["star_in"] = (2101, star, np.zeros_like(star))               # 100 isolated vertices
    a = rng.integers(0, 50, 400).astype(np.uint32)
    b = rng.integers(0, 50, 400).astype(np.uint32)
    out["bridged"] = (200, np.concatenate([a, a + 100, [120]]).astype(np.uint32),
                      np.concatenate([b, b + 100, [7]]).astype(np.uint32))
    return out


def main():
    data = {}
    for name, (V, s, d) in graphs().items():
        data[name + "_V"] = np.uint32(V)
        data[name + "_src"] = np.ascontiguousarray(s, np.uint32)
        data[name + "_dst"] = np.ascontiguousarray(d, np.uint32)
        data[name + "_comp"] = min_labels(V, s, d)
        print(name, V, len(s), "components", len(np.unique(data[name + "_comp"])))
    np.savez_compressed(os.path.join(HERE, "golden_cc.npz"), **data)


if __name__ == "__main__":
    main()
