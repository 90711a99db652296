"""The allocation-free SpMV pull entry point (gg_spmv_pull_noalloc).

Some callers cannot call cudaMalloc: a plugin whose host owns every device
allocation, a real-time loop where an allocation could block, a process whose
device memory is reserved up front.  For them gg_spmv_pull_noalloc runs the
SpMV pull on the caller's own device arrays and keeps its scratch in a fixed
array inside the library.  These tests call it through the C ABI and check
each result against the regular gg_spmv entry point and the oracle with the
floating-point rule the other GPU tests use (tests/fpcheck.py): two calls in
a row on an R-MAT graph, a graph without edges (in_src NULL), a hub whose
row spans many tiles, a call on the legacy default stream, and calls in
contexts that are created, destroyed and reset between calls (the scratch
address must be looked up again in each).  The file is named to be collected
last.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

from fpcheck import assert_fp_as_accurate
from graphs import special_edges

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _bind(gg):
    L = gg.lib()
    L.gg_spmv_pull_noalloc.argtypes = [C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_void_p]
    L.gg_spmv_pull_noalloc.restype = C.c_int
    L.gg_spmv_pull_noalloc_max_items.restype = C.c_uint64
    return L


def _device_arrays(torch, a):
    dev = torch.device("cuda", 0)
    d_off = torch.from_numpy(a["in_off"].view(np.int32).copy()).to(dev)
    d_src = torch.from_numpy(a["in_adj"].view(np.int32).copy()).to(dev) if len(a["in_adj"]) else None
    d_w = torch.from_numpy(a["in_w"].copy()).to(dev) if len(a["in_w"]) else torch.zeros(1, device=dev)
    return d_off, d_src, d_w


def _check_against_gg_spmv(gpu, orc, L, g, x_list, stream_ptr):
    import torch

    a = g.arrays()
    V, E = g.V, g.E
    assert V + E <= L.gg_spmv_pull_noalloc_max_items()
    o = orc.Csr.from_arrays(V, E, a["out_off"], a["out_adj"], a["in_off"], a["in_adj"], a["out_w"], a["in_w"])
    d_off, d_src, d_w = _device_arrays(torch, a)
    d_y = torch.full((V,), float("nan"), dtype=torch.float32, device="cuda")
    dg = gpu.DeviceGraph(g, gpu.MAP_IN | gpu.MAP_IN_W)
    free_after = []
    for call, x in enumerate(x_list):
        d_x = torch.from_numpy(x).cuda()
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        st = L.gg_spmv_pull_noalloc(V, E, d_off.data_ptr(), d_src.data_ptr() if d_src is not None else None,
                                    d_w.data_ptr(), d_x.data_ptr(), d_y.data_ptr(), stream_ptr)
        assert st == 0, gpu.lib().gg_last_error().decode()
        torch.cuda.synchronize()
        free_after.append((free_before, torch.cuda.mem_get_info()[0]))
        y_new = d_y.cpu().numpy()
        _, y_old, _ = dg.spmv("pull", iterations=1, x=x)
        _, y32, _ = orc.spmv(o, 0, 1, x=x)
        y64 = orc.spmv_f64(o, x)
        assert_fp_as_accurate(y_new, y_old, y64, f"call {call} vs gg_spmv")
        assert_fp_as_accurate(y_new, y32, y64, f"call {call} vs the reference's FP32 loop")
    dg.free()
    # the call itself takes no device memory (the first call in a process
    # may load the module; later calls must leave free memory unchanged)
    for before, after in free_after[1:]:
        assert before == after, f"free device memory changed across the call: {before} -> {after}"


def test_spmv_pull_noalloc_matches_gg_spmv_twice(gpu, orc):
    import torch

    L = _bind(gpu)
    g = gpu.Graph.rmat(14, 16, weighted=True)
    rng = np.random.default_rng(5)
    xs = [rng.random(g.V).astype(np.float32) for _ in range(3)]
    _check_against_gg_spmv(gpu, orc, L, g, xs, torch.cuda.current_stream().cuda_stream)


def test_spmv_pull_noalloc_edge_cases(gpu, orc):
    """A graph without edges (in_src NULL, y all zero), a hub with 9000
    in-edges spanning many tiles, and the legacy default stream (NULL)."""
    L = _bind(gpu)
    rng = np.random.default_rng(11)
    sp = special_edges()
    for name in ("no_edges", "hubs"):
        src, dst, w, V = sp[name]
        if w is None:
            w = rng.random(len(src)).astype(np.float32)
        g = gpu.Graph.from_edges(src, dst, w, num_vertices=V)
        xs = [rng.random(g.V).astype(np.float32) for _ in range(2)]
        _check_against_gg_spmv(gpu, orc, L, g, xs, None)
        g.free()


def test_spmv_pull_noalloc_rejects_bad_arguments(gpu):
    L = _bind(gpu)
    limit = int(L.gg_spmv_pull_noalloc_max_items())
    V = 1 << 20
    E = limit - V + 1
    # rejected on the host before any device array is touched
    st = L.gg_spmv_pull_noalloc(V, E, 1, 1, 1, 1, 1, None)
    assert st == 1  # GG_ERR_INVALID
    assert b"exceeds the scratch limit" in gpu.lib().gg_last_error()
    # y overlapping x (aliasing) is rejected, nothing is launched
    base = 1 << 40
    st = L.gg_spmv_pull_noalloc(16, 16, base, base + 4096, base + 8192, base + 12288, base + 12288 + 8, None)
    assert st == 1
    assert b"overlaps" in gpu.lib().gg_last_error()


def test_spmv_pull_noalloc_across_contexts():
    """In a fresh process: a call in the primary context, in a created
    context, in a second created context after the first was destroyed, and
    in the primary context again after it was reset (its module reloaded, the
    scratch at a new address).  Each result is checked against the FP64
    product with the floating-point rule."""
    env = dict(os.environ)
    env["PYTHONPATH"] = os.pathsep.join([os.path.dirname(HERE), HERE, env.get("PYTHONPATH", "")])
    r = subprocess.run([sys.executable, os.path.join(HERE, "noalloc_contexts.py")], env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert "contexts ok" in r.stdout, r.stdout[-3000:]
