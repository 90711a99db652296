"""SpMV on the GPU vs the oracle and the reference's golden vectors.

Tolerances: FP32 pull/push must be at least as accurate against the FP64
oracle as the reference's own FP32 loop (tests/fpcheck.py); fixed-point
modes (2, 3) bit-exact; BF16 / FP16
storage of x and weights vs the FP64 oracle: L1 relative <= 1e-2 / 2e-3.
The reference's SPMVPullFixedPointGraphCSR returns zeros (it reads y from a
local array the FPGA is never given, SPMV.c:900, :980-983); the GPU computes
the fixed-point product the compute unit performs, so mode 2 is compared with
the oracle, not with that golden output.
"""
import os

import numpy as np
import pytest

from fpcheck import assert_fp_as_accurate
from graphs import GOLDEN, fixture_edges, pair, special_edges

pytestmark = pytest.mark.gpu


def _f64(orc, o, x, mode, iters):
    y = orc.spmv_f64(o, x)
    return y * iters if mode == 1 else y


@pytest.fixture(scope="module")
def graphs(gpu, orc):
    out = {}
    for name, (s, d, w) in fixture_edges().items():
        out[name] = pair(gpu, orc, gpu.Graph.from_edges(s, d, w))
        out[name + "_unw"] = pair(gpu, orc, gpu.Graph.from_edges(s, d, None))
    for name, (s, d, w, V) in special_edges().items():
        out[name] = pair(gpu, orc, gpu.Graph.from_edges(s, d, w, num_vertices=V))
    out["rmat10"] = pair(gpu, orc, gpu.Graph.rmat(10, 16, weighted=True))
    out["rmat16w"] = pair(gpu, orc, gpu.Graph.rmat(16, 16, weighted=True))
    out["rmat8_unw"] = pair(gpu, orc, gpu.Graph.rmat(8, 8))
    out["rmat10_unw"] = pair(gpu, orc, gpu.Graph.rmat(10, 16))
    out["rmat12u_unw"] = pair(gpu, orc, gpu.Graph.rmat(12, 8, symmetric=True))
    return out


@pytest.fixture(scope="module")
def dgs(gpu, graphs):
    return {k: gpu.DeviceGraph(g, gpu.MAP_ALL) for k, (g, _) in graphs.items()}


@pytest.mark.parametrize("mode", [0, 1, 2, 3])
def test_spmv_modes_vs_oracle(graphs, dgs, orc, mode):
    for name, (g, o) in graphs.items():
        x, y, res = dgs[name].spmv(mode, iterations=3)
        rx, ry, chk = orc.spmv(o, mode, 3)
        np.testing.assert_array_equal(x, rx)
        if mode in (2, 3):
            np.testing.assert_array_equal(y.view(np.uint32), ry.view(np.uint32), err_msg=name)
        else:
            assert_fp_as_accurate(y, ry, _f64(orc, o, x, mode, 3), name)


@pytest.mark.parametrize("name", ["graphbrew", "test", "v51_e1021", "v300_e2730", "rmat8", "rmat10", "rmat12u"])
def test_spmv_vs_reference_golden(graphs, dgs, orc, name):
    z = np.load(os.path.join(GOLDEN, f"golden_{name}.npz"))
    key = name + "_unw"
    o = graphs[key][1]
    for mode in (0, 1, 3):
        x, y, _ = dgs[key].spmv(mode, iterations=3)
        np.testing.assert_array_equal(x, z[f"spmv{mode}_x"])
        ry = z[f"spmv{mode}_y"]
        if mode == 3:
            np.testing.assert_array_equal(y, ry)
        else:
            assert_fp_as_accurate(y, ry, _f64(orc, o, x, mode, 3), f"{name} mode {mode}")


# One product w*x with both factors rounded to nearest: relative error at
# most 2^-8 (BF16, 8 significant bits each) or 2^-10 (FP16, 11 bits), for
# normal numbers; FP16 subnormals (below 6.1e-5) err by at most 2^-25
# absolutely.  Weights and x are non-negative here, so a row sum's relative
# error is at most its products' largest, plus the FP32 summation's (2e-4
# covers the longest row of this graph): the bounds below follow, and the
# measured L1 lies well inside them (5.7e-4 for BF16 at R-MAT-24).
@pytest.mark.parametrize("storage,tol", [("bf16", 2.0 ** -8 + 2e-4), ("f16", 2.0 ** -10 + 2e-4)])
@pytest.mark.parametrize("mode", ["pull", "push"])
def test_spmv_low_precision(graphs, dgs, orc, storage, tol, mode):
    g, o = graphs["rmat16w"]
    x, y, _ = dgs["rmat16w"].spmv(mode, storage=storage, iterations=1)
    assert (x >= 0).all() and (g.arrays()["in_w"] >= 0).all()
    ex = orc.spmv_f64(o, x)
    assert np.abs(y - ex).sum() / np.abs(ex).sum() <= tol


def test_spmv_explicit_x_and_checksum(graphs, dgs, orc):
    g, o = graphs["rmat10"]
    xin = np.random.default_rng(1).random(g.V).astype(np.float32)
    x, y, res = dgs["rmat10"].spmv("pull", iterations=2, x=xin)
    np.testing.assert_array_equal(x, xin)
    _, ry, chk = orc.spmv(o, 0, 2, x=xin)
    assert_fp_as_accurate(y, ry, orc.spmv_f64(o, xin), "explicit x")
    assert abs(res["checksum"] - chk) <= 0.01 * g.V * 1e-3 + 1e-6
