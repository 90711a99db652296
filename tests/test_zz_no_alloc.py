"""The allocation-free SpMV pull entry point (gg_spmv_pull_noalloc).

Some callers cannot call cudaMalloc: a plugin whose host owns every device
allocation, a real-time loop where an allocation could block, a process whose
device memory is reserved up front.  For them gg_spmv_pull_noalloc runs the
SpMV pull on the caller's own device arrays and keeps its scratch in a fixed
array inside the library.  This test calls it through the C ABI, twice in a
row, and checks each result against the regular gg_spmv entry point with the
floating-point rule the other GPU tests use (tests/fpcheck.py).  The file is
named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

from fpcheck import assert_fp_as_accurate

pytestmark = pytest.mark.gpu


def _bind(gg):
    L = gg.lib()
    L.gg_spmv_pull_noalloc.argtypes = [C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_void_p]
    L.gg_spmv_pull_noalloc.restype = C.c_int
    L.gg_spmv_pull_noalloc_max_items.restype = C.c_uint64
    return L


def test_spmv_pull_noalloc_matches_gg_spmv_twice(gpu, orc):
    import torch

    L = _bind(gpu)
    g = gpu.Graph.rmat(14, 16, weighted=True)
    a = g.arrays()
    V, E = g.V, g.E
    assert V + E <= L.gg_spmv_pull_noalloc_max_items()
    o = orc.Csr.from_arrays(V, E, a["out_off"], a["out_adj"], a["in_off"], a["in_adj"], a["out_w"], a["in_w"])
    dev = torch.device("cuda", 0)
    d_off = torch.from_numpy(a["in_off"].view(np.int32).copy()).to(dev)
    d_src = torch.from_numpy(a["in_adj"].view(np.int32).copy()).to(dev)
    d_w = torch.from_numpy(a["in_w"].copy()).to(dev)
    d_y = torch.empty(V, dtype=torch.float32, device=dev)
    dg = gpu.DeviceGraph(g, gpu.MAP_IN | gpu.MAP_IN_W)
    stream = torch.cuda.current_stream(dev)
    rng = np.random.default_rng(5)
    for call in range(2):
        x = rng.random(V).astype(np.float32)
        d_x = torch.from_numpy(x).to(dev)
        st = L.gg_spmv_pull_noalloc(V, E, d_off.data_ptr(), d_src.data_ptr(), d_w.data_ptr(), d_x.data_ptr(),
                                    d_y.data_ptr(), stream.cuda_stream)
        assert st == 0, gpu.lib().gg_last_error().decode()
        torch.cuda.synchronize()
        y_new = d_y.cpu().numpy()
        _, y_old, _ = dg.spmv("pull", iterations=1, x=x)
        _, y32, _ = orc.spmv(o, 0, 1, x=x)
        y64 = orc.spmv_f64(o, x)
        assert_fp_as_accurate(y_new, y_old, y64, f"call {call} vs gg_spmv")
        assert_fp_as_accurate(y_new, y32, y64, f"call {call} vs the reference's FP32 loop")
    dg.free()


def test_spmv_pull_noalloc_rejects_oversized_graphs(gpu):
    L = _bind(gpu)
    limit = int(L.gg_spmv_pull_noalloc_max_items())
    V = 1 << 20
    E = limit - V + 1
    # rejected on the host before any device array is touched
    st = L.gg_spmv_pull_noalloc(V, E, 1, 1, 1, 1, 1, None)
    assert st == 1  # GG_ERR_INVALID
    assert b"exceeds the scratch limit" in gpu.lib().gg_last_error()
