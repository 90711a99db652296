"""Helper process for tests/test_zz_no_alloc.py (not collected by pytest).

gg_spmv_pull_noalloc looks up its scratch array's device address in the
context current at each call.  This process drives the call from the CUDA
driver API, without torch, through three contexts of device 0:

1. the primary context;
2. a context created with cuCtxCreate (a caller that keeps its own context:
   the library's kernels are loaded into it on the first call and the
   scratch array has another address there);
3. the primary context again, then once more after the created context was
   destroyed.

Every call's y is checked against the oracle's FP64 product with the rule of
tests/fpcheck.py.  Prints "contexts ok" on success.
"""
import ctypes as C
import sys

import numpy as np

import accelgraph_express_gb300 as gg
from fpcheck import assert_fp_as_accurate
from oracle import oracle_ctypes as O

cuda = C.CDLL("libcuda.so.1")
CUdeviceptr = C.c_uint64


def chk(r, what):
    if r != 0:
        raise RuntimeError(f"{what}: CUresult {r}")


class Arrays:
    """The graph's CSC arrays, x and y, allocated in the current context."""

    def __init__(self, o, x):
        self.ptrs = []
        self.in_off = self.put(o.in_off)
        self.in_src = self.put(o.in_adj[:o.E])
        self.w = self.put(o.in_w[:o.E])
        self.x = self.put(x)
        self.y = self.alloc(4 * o.V)

    def alloc(self, n):
        p = CUdeviceptr()
        chk(cuda.cuMemAlloc_v2(C.byref(p), C.c_size_t(max(n, 16))), "cuMemAlloc")
        self.ptrs.append(p)
        return p.value

    def put(self, a):
        a = np.ascontiguousarray(a)
        p = self.alloc(a.nbytes)
        chk(cuda.cuMemcpyHtoD_v2(CUdeviceptr(p), a.ctypes.data_as(C.c_void_p), C.c_size_t(a.nbytes)), "HtoD")
        return p

    def free(self):
        for p in self.ptrs:
            chk(cuda.cuMemFree_v2(p), "cuMemFree")
        self.ptrs = []


def run_once(L, o, x, what):
    a = Arrays(o, x)
    st = L.gg_spmv_pull_noalloc(o.V, o.E, a.in_off, a.in_src, a.w, a.x, a.y, None)
    if st != 0:
        raise RuntimeError(f"{what}: status {st}: {L.gg_last_error().decode()}")
    chk(cuda.cuCtxSynchronize(), "cuCtxSynchronize")
    y = np.empty(o.V, np.float32)
    chk(cuda.cuMemcpyDtoH_v2(y.ctypes.data_as(C.c_void_p), CUdeviceptr(a.y), C.c_size_t(y.nbytes)), "DtoH")
    a.free()
    _, y32, _ = O.spmv(o, 0, 1, x=x)
    assert_fp_as_accurate(y, y32, O.spmv_f64(o, x), what)
    print(what, "ok", flush=True)


def create_context(dev):
    ctx = C.c_void_p()
    if hasattr(cuda, "cuCtxCreate_v2"):
        chk(cuda.cuCtxCreate_v2(C.byref(ctx), C.c_uint(0), dev), "cuCtxCreate")
    else:
        chk(cuda.cuCtxCreate_v4(C.byref(ctx), None, C.c_uint(0), dev), "cuCtxCreate")
    return ctx


def main():
    L = gg.lib()
    L.gg_spmv_pull_noalloc.argtypes = [C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_void_p]
    L.gg_spmv_pull_noalloc.restype = C.c_int
    o = O.rmat_csr(12, 16, weighted=True)
    rng = np.random.default_rng(3)

    chk(cuda.cuInit(0), "cuInit")
    dev = C.c_int()
    chk(cuda.cuDeviceGet(C.byref(dev), 0), "cuDeviceGet")
    primary = C.c_void_p()
    chk(cuda.cuDevicePrimaryCtxRetain(C.byref(primary), dev), "cuDevicePrimaryCtxRetain")
    chk(cuda.cuCtxSetCurrent(primary), "cuCtxSetCurrent")
    run_once(L, o, rng.random(o.V).astype(np.float32), "primary context")

    own = create_context(dev)  # pushed: current on this thread
    run_once(L, o, rng.random(o.V).astype(np.float32), "created context")
    run_once(L, o, rng.random(o.V).astype(np.float32), "created context, second call")
    popped = C.c_void_p()
    chk(cuda.cuCtxPopCurrent_v2(C.byref(popped)), "cuCtxPopCurrent")
    chk(cuda.cuCtxSetCurrent(primary), "cuCtxSetCurrent")
    run_once(L, o, rng.random(o.V).astype(np.float32), "primary context again")
    chk(cuda.cuCtxDestroy_v2(own), "cuCtxDestroy")
    run_once(L, o, rng.random(o.V).astype(np.float32), "primary context after the created one was destroyed")
    chk(cuda.cuDevicePrimaryCtxRelease_v2(dev), "cuDevicePrimaryCtxRelease")
    print("contexts ok", flush=True)


if __name__ == "__main__":
    sys.exit(main())
