"""Test graphs shared by the parity tests: the product's Graph and the
oracle's view of the same arrays."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def pair(gg, O, graph):
    a = graph.arrays()
    o = O.Csr.from_arrays(graph.V, graph.E, a["out_off"], a["out_adj"], a["in_off"], a["in_adj"],
                          a["out_w"], a["in_w"])
    return graph, o


def fixture_edges():
    """The reference's fixture graphs (04_test_graphs/TEST), as stored in
    tests/golden/fixtures.npz."""
    z = np.load(os.path.join(GOLDEN, "fixtures.npz"))
    out = {}
    for name in ["graphbrew", "test", "v51_e1021", "v300_e2730"]:
        w = z[name + "_w"] if name + "_w" in z.files else None
        out[name] = (z[name + "_src"], z[name + "_dst"], w)
    return out


def special_edges():
    """Edge cases: a hub whose in- and out-lists span many merge-path tiles,
    isolated vertices, self loops, duplicates, a chain, a single edge, a
    directed ring (4096 levels from any source, every contribution equal:
    direction-optimised BFS drains its edge budget one edge per level and
    turns bottom-up near the end), and a graph without edges."""
    rng = np.random.default_rng(7)
    V = 5000
    hub_in = np.stack([rng.integers(0, V, 9000), np.zeros(9000, np.int64)], 1)      # in-degree 9000 at 0
    hub_out = np.stack([np.full(7000, 3), rng.integers(0, V, 7000)], 1)              # out-degree 7000 at 3
    loops = np.stack([np.arange(10, 20), np.arange(10, 20)], 1)                      # self loops
    dups = np.array([[5, 6]] * 40)                                                   # duplicates
    chain = np.stack([np.arange(100, 400), np.arange(101, 401)], 1)                  # long chain
    e = np.concatenate([hub_in, hub_out, loops, dups, chain]).astype(np.uint32)
    return {
        "hubs": (e[:, 0], e[:, 1], rng.random(len(e)).astype(np.float32), V + 50),  # 50 isolated
        "single": (np.array([0], np.uint32), np.array([1], np.uint32), None, 2),
        "star_out": (np.zeros(4000, np.uint32), np.arange(1, 4001, dtype=np.uint32), None, 4001),
        "star_in": (np.arange(1, 4001, dtype=np.uint32), np.zeros(4000, np.uint32), None, 4001),
        "ring": (np.arange(4096, dtype=np.uint32), (np.arange(1, 4097) % 4096).astype(np.uint32), None, 4096),
        "no_edges": (np.zeros(0, np.uint32), np.zeros(0, np.uint32), None, 64),
    }
