"""bench.py's reference arm (the CPU implementation of the path) runs without
a GPU and prints one JSON line with every key of the benchmark contract:
the metric line itself, `impl`, a `cpu_baseline` describing the run, and an
`e2e` object with no host-device traffic."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

KEYS = ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
        "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e")


def test_reference_arm_prints_the_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--scale", "10",
                          "--steps", "2", "--warmup", "1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [x for x in out.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1, out.stdout[-2000:]
    line = json.loads(lines[0])
    for k in KEYS:
        assert k in line, k
    assert line["impl"] == "reference" and line["steps"] == 2 and line["warmup"] == 1
    assert line["value"] > 0 and line["ms_per_step"] > 0 and line["higher_is_better"] is True
    assert "workload" in line["config"]
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert cb["unit"] == line["unit"] and cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_runs_the_same_config_without_the_product():
    """The reference arm times the GPU arm's step (30 iterations) and never
    imports or loads the product library: it builds its graph with the
    oracle."""
    code = ("import runpy, sys; sys.argv = ['bench.py', '--impl', 'reference', '--scale', '9', '--steps', '1', "
            "'--warmup', '0']; runpy.run_path('bench.py', run_name='__main__'); "
            "maps = open('/proc/self/maps').read(); "
            "assert 'accelgraph_express_gb300' not in sys.modules; "
            "assert 'libaccelgraph_gb300' not in maps, 'product library loaded'")
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads([x for x in out.stdout.splitlines() if x.startswith("{")][0])
    assert line["config"]["iterations_per_step"] == 30 and line["config"]["epsilon"] == 0.0
    assert line["config"]["workload"] == "pagerank_pull_rmat9"


def test_algorithmic_bytes_match_the_stated_figures():
    """The byte counts behind roofline.achieved: one PageRank pull iteration
    (4E + 4(V+1) + (12+2s)V) and one gather launch (4E + 4(V+1) + sV + 4V) at
    the R-MAT-24 and R-MAT-16 workloads, FP32, and the R-MAT-24 iteration
    with BF16 contributions."""
    sys.path.insert(0, ROOT)
    import bench

    assert bench.pr_bytes(1 << 24, 1 << 28, 4) == 1_476_395_012
    assert bench.pr_bytes(1 << 16, 1 << 20, 4) == 5_767_172
    assert bench.pr_gather_bytes(1 << 24, 1 << 28, 4) == 1_275_068_420
    assert bench.pr_bytes(1 << 24, 1 << 28, 2) == 1_409_286_148
