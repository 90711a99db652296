"""Connected components on the GPU against the golden labels (smallest id of
each weakly connected component, tests/golden/golden_cc.npz) and the oracle:
bit-exact labels for all three algorithms (Shiloach-Vishkin, Afforest,
weakly connected components), through gg_cc and the reference's drop-in
entry points."""
import os

import ctypes as C

import numpy as np
import pytest

from graphs import GOLDEN, fixture_edges, special_edges

pytestmark = pytest.mark.gpu

Z = np.load(os.path.join(GOLDEN, "golden_cc.npz"))
NAMES = sorted({k.rsplit("_", 1)[0] for k in Z.files})


def _graph(gpu, name):
    V = int(Z[name + "_V"])
    return gpu.Graph.from_edges(Z[name + "_src"], Z[name + "_dst"], num_vertices=V), Z[name + "_comp"]


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("algorithm", ["sv", "afforest", "weakly"])
def test_cc_matches_golden(gpu, name, algorithm):
    g, gold = _graph(gpu, name)
    dg = gpu.DeviceGraph(g, gpu.MAP_OUT | gpu.MAP_IN)
    comp, r = dg.cc(algorithm)
    np.testing.assert_array_equal(comp, gold, err_msg=f"{name} {algorithm}")
    assert r["components"] == len(np.unique(gold))
    assert r["iterations"] >= 1


@pytest.mark.parametrize("samples", [1, 7, 1024])
def test_cc_afforest_any_sample(gpu, samples):
    """The sample only picks which component skips the final link."""
    g, gold = _graph(gpu, "rmat14")
    dg = gpu.DeviceGraph(g, gpu.MAP_OUT | gpu.MAP_IN)
    for seed in (1, 2, 3):
        comp, r = dg.cc("afforest", samples=samples, seed=seed)
        np.testing.assert_array_equal(comp, gold)


def test_cc_afforest_symmetric_out_edges_only(gpu):
    """Declared symmetric, Afforest links out-edges only (no CSC needed)."""
    g, gold = _graph(gpu, "rmat12u")
    dg = gpu.DeviceGraph(g, gpu.MAP_OUT)
    comp, r = dg.cc("afforest", use_in_edges=0)
    np.testing.assert_array_equal(comp, gold)
    # without the CSC and without the symmetric promise nothing is skipped
    comp, r = dg.cc("afforest", use_in_edges=2)
    np.testing.assert_array_equal(comp, gold)
    assert r["skipped_label"] == 0xFFFFFFFF


@pytest.mark.parametrize("symmetric", [False, True])
def test_cc_rmat18_vs_oracle(gpu, orc, symmetric):
    g = gpu.Graph.rmat(18, 8, symmetric=symmetric)
    a = g.arrays()
    o = orc.Csr.from_arrays(g.V, g.E, a["out_off"], a["out_adj"], a["in_off"], a["in_adj"])
    gold = orc.cc_min_label(o)
    dg = gpu.DeviceGraph(g, gpu.MAP_OUT | gpu.MAP_IN)
    for algorithm in ("sv", "afforest", "weakly"):
        comp, _ = dg.cc(algorithm)
        np.testing.assert_array_equal(comp, gold, err_msg=algorithm)


@pytest.mark.parametrize("pushpull", [0, 1, 2, 3])
def test_cc_dropin(gpu, pushpull):
    """connectedComponentsGraphCSR dispatches on pushpull (3 -> Afforest);
    counts and labels are left as the reference's printCCStats leaves them
    (sizes ascending, the label of each beside it, ties by ascending id);
    the host verify passes."""
    gpu.set_gpu_options(keep_resident=False, verbose=False)
    for name in ("v300_e2730", "rmat14", "bridged"):
        g, gold = _graph(gpu, name)
        args = gpu.default_arguments()
        args.pushpull = pushpull
        comp, counts, labels, info, ok = gpu.cc_csr(g, args, verify=True)
        np.testing.assert_array_equal(comp, gold, err_msg=name)
        # Afforest (pushpull 1 and the default) advances the caller's
        # generator by its sample count, as the reference's sampling does
        fresh = gpu.default_arguments()
        draws = (1024 if g.V >= 1024 else g.V // 2) if pushpull in (1, 3) else 0
        for _ in range(draws):
            gpu.lib().generateRandInt(C.byref(fresh.mt19937var))
        assert bytes(fresh.mt19937var) == bytes(args.mt19937var), name
        size = np.bincount(gold, minlength=g.V).astype(np.uint32)
        order = np.argsort(size, kind="stable")
        np.testing.assert_array_equal(labels, order.astype(np.uint32), err_msg=name)
        np.testing.assert_array_equal(counts, size[order], err_msg=name)
        assert ok == 1
        assert info["neighbor_rounds"] == 2
        if pushpull in (1, 3):
            assert info["iterations"] == 0  # the reference's Afforest never counts them
        else:
            assert info["iterations"] >= 1


REF_NAMES = ["graphbrew", "test", "v51_e1021", "v300_e2730", "rmat8", "rmat10", "rmat12u",
             "hubs", "single", "star_out", "star_in", "ring", "no_edges"]
REF_RMAT = {"rmat8": (8, 8, False), "rmat10": (10, 16, False), "rmat12u": (12, 8, True)}


def _ref_graph(gpu, name):
    if name in REF_RMAT:
        s, e, sym = REF_RMAT[name]
        return gpu.Graph.rmat(s, e, weighted=True, symmetric=sym)
    special = special_edges()
    if name in special:
        s, d, w, V = special[name]
        return gpu.Graph.from_edges(s, d, w, num_vertices=V)
    s, d, w = fixture_edges()[name]
    return gpu.Graph.from_edges(s, d, w)


@pytest.mark.parametrize("name", REF_NAMES)
def test_cc_dropin_vs_reference_golden(gpu, name):
    """Against outputs of the reference's own connectedComponents.c
    (tests/golden/make_golden.py): for Afforest (pushpull 1) and weakly (2)
    the drop-in leaves the same components, counts and labels, Afforest's
    iteration count, and the caller's generator in the same state."""
    gpu.set_gpu_options(keep_resident=False, verbose=False)
    z = np.load(os.path.join(GOLDEN, f"golden_{name}.npz"))
    g = _ref_graph(gpu, name)
    assert int(z["V"]) == g.V and int(z["E"]) == g.E
    for pushpull in (1, 2):
        args = gpu.default_arguments()
        args.pushpull = pushpull
        comp, counts, labels, info = gpu.cc_csr(g, args)
        tag = f"{name} pushpull {pushpull}"
        np.testing.assert_array_equal(comp, z[f"cc{pushpull}_components"], err_msg=tag)
        np.testing.assert_array_equal(counts, z[f"cc{pushpull}_counts"], err_msg=tag)
        np.testing.assert_array_equal(labels, z[f"cc{pushpull}_labels"], err_msg=tag)
        if pushpull == 1:
            assert info["iterations"] == int(z["cc1_iterations"]), tag
        np.testing.assert_array_equal(np.frombuffer(bytes(args.mt19937var), np.uint32), z[f"cc{pushpull}_mt"],
                                      err_msg=tag)


def test_cc_named_entry_points(gpu):
    g, gold = _graph(gpu, "rmat10")
    args = gpu.default_arguments()
    for fn in ("connectedComponentsShiloachVishkinGraphCSR", "connectedComponentsAfforestGraphCSR",
               "connectedComponentsWeaklyGraphCSR"):
        comp, _, _, _ = gpu.cc_csr(g, args, fn=fn)
        np.testing.assert_array_equal(comp, gold, err_msg=fn)


@pytest.mark.parametrize("algorithm", ["sv", "afforest", "weakly"])
def test_cc_no_edges(gpu, algorithm):
    """Every vertex is its own component."""
    g = gpu.Graph.from_edges(np.zeros(0, np.uint32), np.zeros(0, np.uint32), num_vertices=100)
    dg = gpu.DeviceGraph(g, gpu.MAP_OUT | gpu.MAP_IN)
    comp, r = dg.cc(algorithm)
    np.testing.assert_array_equal(comp, np.arange(100, dtype=np.uint32))
    assert r["components"] == 100


def test_cc_invalid(gpu):
    g, _ = _graph(gpu, "rmat10")
    dg = gpu.DeviceGraph(g, gpu.MAP_IN)
    with pytest.raises(gpu.GgError):
        dg.cc("sv")  # needs the out-CSR
    dg2 = gpu.DeviceGraph(g, gpu.MAP_OUT)
    with pytest.raises(gpu.GgError):
        dg2.cc(7)
