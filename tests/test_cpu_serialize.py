"""Graph files: the reference's -z / -c / -x options (02_capi_graph/src/main/
accel-graph.c:51, :115-128, :339-341) on the CPU.

* text and binary edge lists written and read back give the same edges;
* a graphCSR binary file read back gives a graph whose every array equals
  the written graph's (the layout is this project's own: OpenGraph, which
  defines the reference's, is absent);
* writeSerializedGraphDataStructure converts between the three formats as
  -x -c does, and the converted files load into the same CSR;
* where the reference tree is present, writing the fixture edge lists
  reproduces the reference's own 04_test_graphs files byte for byte.
"""
import ctypes as C
import os

import numpy as np
import pytest

from graphs import fixture_edges, special_edges

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KEYS = ("out_off", "out_adj", "in_off", "in_adj", "out_degree", "in_degree", "out_w", "in_w")


def _graphs(gg):
    out = {}
    for name, (s, d, w) in fixture_edges().items():
        out[name] = gg.Graph.from_edges(s, d, w)
    for name, (s, d, w, V) in special_edges().items():
        out[name] = gg.Graph.from_edges(s, d, w, num_vertices=V)
    out["rmat10w"] = gg.Graph.rmat(10, 8, weighted=True)
    out["rmat12u"] = gg.Graph.rmat(12, 4, symmetric=True)
    return out


def _same(a, b):
    for k in KEYS:
        if a[k] is None or b[k] is None:
            assert a[k] is None and b[k] is None, k
        else:
            np.testing.assert_array_equal(a[k], b[k], err_msg=k)


def _labels_and_rows(gg, g):
    e, ie = g.ptr.contents.sorted_edges_array.contents, g.ptr.contents.inverse_sorted_edges_array.contents
    return [gg._np(p, n, np.uint32) for p, n in ((e.edges_array_src, g.E), (ie.edges_array_src, g.E),
                                                   (e.label_array, g.V), (e.inverse_label_array, g.V),
                                                   (ie.label_array, g.V), (ie.inverse_label_array, g.V))]


def test_graphcsr_binary_round_trip(gg, tmp_path):
    for name, g in _graphs(gg).items():
        path = str(tmp_path / f"{name}.csr")
        g.save(path)
        h = gg.Graph.from_file(path)
        assert (h.V, h.E) == (g.V, g.E), name
        assert h.ptr.contents.max_weight == g.ptr.contents.max_weight
        assert h.ptr.contents.avg_degree == g.ptr.contents.avg_degree
        _same(g.arrays(), h.arrays())
        for x, y in zip(_labels_and_rows(gg, g), _labels_and_rows(gg, h)):
            np.testing.assert_array_equal(x, y)


def test_edge_list_round_trips(gg, tmp_path):
    for name, g in _graphs(gg).items():
        w = g.arrays()["out_w"]
        weighted = w is not None
        for binary in (False, True):
            if binary and weighted and not np.array_equal(w, np.round(w)):
                continue  # fractional weights: the .wbin weight word is an integer
            path = str(tmp_path / (f"{name}.wbin" if weighted else f"{name}.bin") if binary
                       else tmp_path / f"{name}.txt")
            g.save_edges(path, binary=binary)
            h = gg.Graph.from_file(path, weighted=weighted)
            if g.E == 0:
                assert h.E == 0
                continue
            # the loaders take V = max id + 1, so isolated tail vertices are dropped
            a, b = g.arrays(), h.arrays()
            np.testing.assert_array_equal(a["out_adj"], b["out_adj"], err_msg=name)
            np.testing.assert_array_equal(a["in_adj"], b["in_adj"], err_msg=name)
            np.testing.assert_array_equal(a["out_off"][:h.V + 1], b["out_off"], err_msg=name)
            if weighted:
                np.testing.assert_array_equal(a["out_w"], b["out_w"], err_msg=name)


def test_integer_weights_round_trip_through_wbin(gg, tmp_path):
    s, d, w = fixture_edges()["v51_e1021"]
    assert w is not None and np.array_equal(w, np.round(w))
    g = gg.Graph.from_edges(s, d, w)
    g.save_edges(str(tmp_path / "g.wbin"))
    _same(g.arrays(), gg.Graph.from_file(str(tmp_path / "g.wbin"), weighted=True).arrays())


def test_serialize_entry_point_converts_between_formats(gg, tmp_path):
    L = gg.lib()
    s, d, w = fixture_edges()["v300_e2730"]
    src = tmp_path / "g.wbin"
    np.stack([s, d, w.astype(np.uint32)], 1).astype(np.uint32).tofile(src)
    ref = gg.Graph.from_file(str(src), weighted=True).arrays()
    args = gg.default_arguments()
    path = str(src).encode()
    args.fnameb = path
    args.weighted = 1
    # -z 1 -c 2: binary edge list -> graphCSR binary
    args.fnameb_format, args.convert_format = 1, 2
    L.writeSerializedGraphDataStructure(C.byref(args))
    _same(ref, gg.Graph.from_file(str(src) + ".csr").arrays())
    # -z 1 -c 0: -> text edge list
    args.convert_format = 0
    L.writeSerializedGraphDataStructure(C.byref(args))
    _same(ref, gg.Graph.from_file(str(src) + ".txt", weighted=True).arrays())
    # -z 2 -c 1: graphCSR binary -> binary edge list (CSR order)
    csr = str(src) + ".csr"
    args.fnameb, args.fnameb_format, args.convert_format = csr.encode(), 2, 1
    L.writeSerializedGraphDataStructure(C.byref(args))
    _same(ref, gg.Graph.from_file(csr + ".wbin", weighted=True).arrays())


def test_bad_files_are_rejected(gg, tmp_path):
    L = gg.lib()
    bad = tmp_path / "bad.csr"
    bad.write_bytes(b"not a graph file at all, just some bytes......")
    assert not L.readGraphCSRbin(str(bad).encode())
    g = gg.Graph.rmat(6, 4)
    g.save(str(tmp_path / "t.csr"))
    data = (tmp_path / "t.csr").read_bytes()
    (tmp_path / "short.csr").write_bytes(data[:-4])
    assert not L.readGraphCSRbin(str(tmp_path / "short.csr").encode())
    assert not L.readGraphCSRbin(str(tmp_path / "missing.csr").encode())


def _reference_test_graphs():
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(ROOT, "tests", "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg.TEST if os.path.isdir(mg.TEST) else None, mg.FIXTURES


def test_fixture_files_written_back_byte_for_byte(gg, tmp_path):
    """The fixture edge lists (read from the reference's files) written with
    writeEdgeListsbin equal the reference's own .bin / .wbin files."""
    test_dir, files = _reference_test_graphs()
    if test_dir is None:
        pytest.skip("reference tree not present")
    L = gg.lib()
    for name, (s, d, w) in fixture_edges().items():
        rel, weighted = files[name]
        el = gg.Graph._edge_list(s, d, w if weighted else None)
        try:
            out = str(tmp_path / os.path.basename(rel))
            assert L.writeEdgeListsbin(el, out.encode()) == 0
        finally:
            L.freeEdgeList(el)
        with open(os.path.join(test_dir, rel), "rb") as f:
            assert open(out, "rb").read() == f.read(), name
