"""The C caller of INTEGRATION.md section 2, compiled with gcc against
include/ and linked to libaccelgraph_gb300.so, run on the reference's
v300_e2730 fixture (written as a .wbin file): its printed PageRank, BFS,
SpMV and connected-components results are checked against the oracle --
PageRank iterations and BFS processed vertices exact, the first rank and
the first SpMV output within 1e-5 relative of the oracle's FP32 values,
and the components verified by the library's own check.
"""
import os
import re
import subprocess

import numpy as np
import pytest

from graphs import fixture_edges

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _snippet():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    sec = text[text.index("## 2. Call sites"):]
    m = re.search(r"```c\n(.*?)```", sec, re.S)
    assert m, "no C block in section 2"
    return m.group(1)


def test_integration_c_caller_builds_and_matches_the_oracle(gpu, orc, tmp_path):
    src = tmp_path / "pr_bfs_cc.c"
    src.write_text(_snippet())
    libdir = os.path.dirname(gpu.LIB_PATH)
    exe = tmp_path / "pr_bfs_cc"
    cc = subprocess.run(["gcc", "-std=gnu11", "-O1", "-Wall", str(src), "-I", os.path.join(ROOT, "include"),
                         "-L", libdir, "-laccelgraph_gb300", f"-Wl,-rpath,{libdir}", "-o", str(exe)],
                        capture_output=True, text=True)
    assert cc.returncode == 0, cc.stderr
    s, d, w = fixture_edges()["v300_e2730"]
    path = tmp_path / "graph.wbin"
    np.stack([s, d, w.astype(np.uint32)], 1).astype(np.uint32).tofile(path)
    run = subprocess.run([str(exe), str(path)], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout[-2000:] + run.stderr[-2000:]
    out = run.stdout
    V = int(max(s.max(), d.max())) + 1
    o = orc.Csr(V, s, d, w)
    ranks, info = orc.pagerank(o, 0, 20, 1e-4)
    m = re.search(r"pagerank iterations (\d+) rank0 (\S+)", out)
    assert m and int(m.group(1)) == info["iterations"], out
    assert abs(float(m.group(2)) - ranks[0]) <= 1e-5 * abs(ranks[0]), (m.group(2), ranks[0])
    _, _, binfo = orc.bfs(o, 2, 0)
    m = re.search(r"bfs processed (\d+)", out)
    assert m and int(m.group(1)) == binfo["processed_nodes"], out
    _, y, _ = orc.spmv(o, 0, 1)
    m = re.search(r"spmv y0 (\S+)", out)
    assert m and abs(float(m.group(1)) - y[0]) <= 1e-5 * max(abs(y[0]), 1e-30), (m.group(1), y[0])
    assert "components verified" in out
