#!/usr/bin/env python3
"""Benchmark: PageRank pull on a directed R-MAT scale-24 graph (16.7M vertices,
268M edges, a,b,c,d = 0.57/0.19/0.19/0.05, seed 27491095), FP32, 30
iterations per step, in GTEPS (edges x iterations / second).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

value      GTEPS with the graph resident in HBM, device time (CUDA events on
           the launching stream) over exactly K steps, max over ranks.
e2e        the same metric through the drop-in pageRankGraphCSR call on host
           arrays: every step uploads the CSC (offsets, neighbour ids) and
           out-degrees and reads the ranks back.
roofline   the gather kernel (k_pr_pull_hot from 1M vertices: the pull gather
           with the hot-vertex table; k_pr_pull below): algorithmic bytes per launch
           4E + 4(V+1) + sV + 4V with s = 4 bytes of FP32 contribution (CSC
           ids, CSC offsets, each contribution once, the row sums written),
           / its mean CUDA-event duration, vs the measured HBM copy
           bandwidth; `iteration` rates a whole iteration (gather + vertex
           update) against the algorithm's 4E + 4(V+1) + (12 + 2s)V.
extras     BF16/FP16 PageRank, SpMV pull, BFS (R-MAT-22 undirected, 64
           sources), batched personalised PageRank (K = 64), 4096 graphs in
           one CUDA-graph launch, and the query server under Poisson load.
cpu_baseline  the oracle's OpenMP restatement of the reference's pull loop
           (pageRank.c:1026-1085 with the gather as at :2890-2906) on all host
           cores, on a bounded number of iterations of the same graph.
--impl reference  times that CPU implementation alone on the same graph
           (built by the oracle), 30 iterations per step as this arm's step
           (the reference's own code needs its absent OpenGraph library and
           FPGA, so the restatement stands in for it).
With N > 1 GPUs every rank runs an independent replica (no collective on the
data path); value sums all ranks' edges over the slowest rank's time.
"""
import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SEED = 27491095
ITERS = 30


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--scale", type=int, default=24)
    p.add_argument("--edge-factor", type=int, default=16)
    p.add_argument("--no-extras", action="store_true", help="skip the BF16/BFS/SpMV side measurements")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    p.add_argument("--leg", choices=["pr", "c1", "bfs", "ppr", "batch", "serve", "csr", "cc", "relabel"],
                   help="run one side measurement alone and print its JSON (for profiling)")
    p.add_argument("--leg-scale", type=int,
                   help="R-MAT scale of the --leg graph, or the number of graphs of --leg batch (small cases for profiling)")
    return p.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class Clocks:
    """nvidia-smi samples (200 ms) while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = os.path.join("/tmp", f"bench_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def load_traffic(kernel):
    """dram bytes per launch of `kernel` from the committed ncu summary."""
    try:
        with open(os.path.join(ROOT, "profiles", "roofline_traffic.json")) as f:
            d = json.load(f)
        return d.get(kernel, {}).get("dram_bytes_per_launch")
    except Exception:
        return None


def pr_bytes(V, E, s):
    """Algorithmic bytes of one PageRank pull iteration: CSC ids, offsets,
    and per vertex rank read+write, out-degree, contribution read+write."""
    return 4 * E + 4 * (V + 1) + (12 + 2 * s) * V


def pr_gather_bytes(V, E, s):
    """Algorithmic bytes of one k_pr_pull launch (the gather): CSC ids,
    offsets, each contribution once, and the row sums it writes."""
    return 4 * E + 4 * (V + 1) + s * V + 4 * V


def cpu_pagerank(graph, O, iters, threads):
    """The oracle's OpenMP pull on the product's graph arrays (zero copy)."""
    v = graph.views()
    V, E = graph.V, graph.E
    import numpy as np
    out_off = np.append(v["out_edges_idx"], np.uint32(E))
    in_off = np.append(v["in_edges_idx"], np.uint32(E))
    o = O.Csr.from_arrays(V, E, out_off, v["out_adj"], in_off, v["in_adj"])
    t0 = time.perf_counter()
    ranks, info = O.pagerank(o, 0, iters, 0.0, nthreads=threads)
    dt = time.perf_counter() - t0
    return ranks, info, dt, o


def hold_collector():
    """Collect the Python heap once and switch the cyclic collector off for
    the rest of the run.  Every timed call is a C call or a device launch,
    and a full collection of this process's heap takes ~50 ms once torch is
    imported: landing inside a timed region it is a pause of the harness,
    not of the library (a single 93 ms drop-in call among 37 ms ones matched
    it).  Objects are still freed by reference counting."""
    gc.collect()
    gc.disable()


def run_reference(a, world, rank):
    """The reference arm: the CPU implementation of the path on the host's
    cores, on this arm's own workload and config.  The graph comes from the
    oracle's R-MAT generator and CSR build (the same edges and arrays as the
    product's builder gives; nothing of the product is imported), and every
    step runs the full 30 pull iterations of the GPU arm's step with the
    oracle's OpenMP restatement of the reference's pull loop (pageRank.c:
    1026-1085, gather as at :2890-2906).  The reference's own compiled code
    needs its absent OpenGraph library and its FPGA; the restatement is
    bit-exact with that code compiled against stand-ins where the reference
    tree is mounted."""
    if rank != 0:
        return
    from oracle import oracle_ctypes as O

    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    o = O.rmat_csr(a.scale, a.edge_factor, seed=SEED)
    build_s = time.perf_counter() - t0
    hold_collector()
    V, E = o.V, o.E
    times = []
    for i in range(a.warmup + a.steps):
        t0 = time.perf_counter()
        O.pagerank(o, 0, ITERS, 0.0, nthreads=threads)
        dt = time.perf_counter() - t0
        if i >= a.warmup:
            times.append(dt)
    t = sum(times)
    value = E * ITERS * len(times) / t / 1e9
    line = {
        "impl": "reference", "metric": f"PageRank pull GTEPS, R-MAT-{a.scale} FP32", "value": value,
        "unit": "GTEPS", "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": 1e3 * t / len(times), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32",
        "data": f"synthetic R-MAT scale {a.scale}, edge factor {a.edge_factor}, seed {SEED}, no label permutation",
        "config": {"workload": f"pagerank_pull_rmat{a.scale}", "vertices": V, "edges": E,
                   "iterations_per_step": ITERS, "epsilon": 0.0, "storage": "f32", "threads": threads,
                   "graph_build_s": round(build_s, 2)},
        "cpu_baseline": {"value": value, "unit": "GTEPS", "cores": threads, "kind": "port",
                         "sample": f"{ITERS} PageRank pull iterations over R-MAT-{a.scale} per step, "
                                   f"{a.steps} steps"},
        "e2e": {"value": value, "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


class Replicas:
    """The N > 1 plumbing of the replicas: one process per GPU, each running
    the whole workload on its own graph copy; no collective on the data path,
    only a barrier around the timed region and the max of the ranks' times.
    (backend/device: "nccl"/"cuda" on GPUs; "gloo"/"cpu" in the CPU tests.)"""

    def __init__(self, world, backend="nccl", device="cuda"):
        self.world, self.device, self.dist = world, device, None
        if world > 1:
            import torch.distributed as dist
            if not dist.is_initialized():
                dist.init_process_group(backend)
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, x):
        if not self.dist:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64, device=self.device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()
            self.dist = None

    def value(self, units_per_rank, slowest_ms):
        """Whole-job throughput: every rank's units over the slowest rank's time."""
        return self.world * units_per_rank / (slowest_ms / 1e3)


def run_leg(leg, scale=None):
    """One side measurement alone, its JSON on stdout; `scale` shrinks the
    leg's R-MAT graph (for profiling captures on a small case)."""
    import torch

    import accelgraph_express_gb300 as gg

    gg.device_init(0)
    peak, _ = load_peaks()
    kw = {} if scale is None else {"scale": scale}
    hold_collector()

    def pr():
        g = gg.Graph.rmat(scale or 24, 16, seed=SEED)
        dg = gg.DeviceGraph(g, gg.MAP_IN)
        r = pr_storage_extras(gg, g, dg, g.V, g.E, torch.cuda.current_stream().cuda_stream, torch, peak)
        dg.free()
        return r

    fn = {"pr": pr, "c1": lambda: c1_extras(gg, torch, peak=peak, **kw),
          "bfs": lambda: bfs_extras(gg, torch, peak, **kw), "ppr": lambda: ppr_extras(gg, torch, peak, **kw),
          "batch": lambda: batch_extras(gg, torch, peak, **({} if scale is None else {"n": scale})), "serve": lambda: serving_extras(gg, **kw),
          "csr": lambda: csr_build_extras(gg, torch, peak, **kw), "cc": lambda: cc_extras(gg, torch, peak),
          "relabel": lambda: relabel_extras(gg, torch, peak, **kw)}[leg]
    print(json.dumps({"leg": leg, **fn()}), flush=True)


def main():
    a = parse()
    world, rank, local = dist_env()
    if a.impl == "reference":
        run_reference(a, world, rank)
        return
    if a.leg:
        run_leg(a.leg, a.leg_scale)
        return

    import numpy as np
    import torch

    import accelgraph_express_gb300 as gg

    torch.cuda.set_device(local)
    reps = Replicas(world, "nccl", "cuda")
    barrier, max_over_ranks = reps.barrier, reps.max

    gg.device_init(local)
    t_build = time.perf_counter()
    # one weighted graph serves PageRank (weights unused) and SpMV
    graph = gg.Graph.rmat(a.scale, a.edge_factor, seed=SEED, weighted=not a.no_extras, weight_seed=SEED + 2)
    t_build = time.perf_counter() - t_build
    V, E = graph.V, graph.E
    dg = gg.DeviceGraph(graph, gg.MAP_IN)
    hold_collector()
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    # launch shape of the gather picked by the autotuner on this graph
    # (setup, like the graph build; the default shape is one candidate)
    tune = dg.autotune(gg.TUNE_PR, reps=3, stream=sptr).get("pr")

    def step(profile=True):
        _, r = dg.pagerank("pull", iterations=ITERS, epsilon=0.0, copy_out=False, profile=profile, stream=sptr)
        return r

    for _ in range(a.warmup):
        step()
    torch.cuda.synchronize()

    clocks = Clocks(local)
    clocks.start()
    barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    gather_ms, gather_n, launches, hot = 0.0, 0, 0, 0
    for _ in range(a.steps):
        r = step()
        gather_ms += r["gather_ms"]
        gather_n += r["gather_launches"]
        launches += r["launches"]
        hot = r["hot_table"]
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    elapsed_ms = max_over_ranks(ev0.elapsed_time(ev1))
    value = reps.value(E * ITERS * a.steps, elapsed_ms) / 1e9

    # roofline of the gather kernel
    peak, peak_kind = load_peaks()
    per_launch_ms = gather_ms / max(gather_n, 1)
    alg = pr_gather_bytes(V, E, 4)
    achieved = alg / (per_launch_ms / 1e3) / 1e9
    kernel = "k_pr_pull_hot" if hot else "k_pr_pull"
    traffic = load_traffic(kernel)
    # the whole iteration (gather + vertex update) against the algorithm's bytes
    iter_ms = elapsed_ms / (a.steps * ITERS)
    iteration = {"alg_bytes": pr_bytes(V, E, 4), "ms": iter_ms,
                 "frac": pr_bytes(V, E, 4) / (iter_ms / 1e3) / 1e9 / peak}

    # e2e through the drop-in entry point on host arrays, called as a C
    # caller calls it: pageRankGraphCSR maps the host graph, runs, copies the
    # ranks into the host stats; freePageRankStats releases them
    import ctypes as C

    gg.set_gpu_options(storage="f32", device=local, keep_resident=False, verbose=False)
    args = gg.default_arguments(iterations=ITERS, epsilon=0.0)
    L = gg.lib()

    def dropin_call():
        st = L.pageRankGraphCSR(C.byref(args), graph.ptr)
        if not st:
            raise gg.GgError(f"pageRankGraphCSR failed: {L.gg_last_error().decode()}")
        L.freePageRankStats(st)

    for _ in range(max(3, a.warmup)):
        dropin_call()
    barrier()
    t0 = time.perf_counter()
    # 50 calls (~2 s): a single stall of the shared host (calls of 60-130 ms
    # were seen in long runs, none in 300 calls run alone) moves the mean
    # less than over 20
    e2e_steps = max(3, min(a.steps, 50))
    call_ms = []
    for _ in range(e2e_steps):
        tc = time.perf_counter()
        dropin_call()
        call_ms.append((time.perf_counter() - tc) * 1e3)
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    e2e_value = world * E * ITERS * e2e_steps / e2e_s / 1e9
    h2d = 4 * V + 4 + 4 * E + 4 * V  # CSC edges_idx (+ E sentinel), CSC neighbour ids, out-degree
    d2h = 4 * V + (ITERS + 2) * 16 + 8  # ranks, per-iteration records, rank sum

    line = {
        "metric": f"PageRank pull GTEPS, R-MAT-{a.scale} FP32", "value": value, "unit": "GTEPS",
        "n_gpus": world, "steps": a.steps, "warmup": a.warmup, "ms_per_step": elapsed_ms / a.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": f"synthetic R-MAT scale {a.scale}, edge factor {a.edge_factor}, seed {SEED}, no label permutation",
        "config": {"workload": f"pagerank_pull_rmat{a.scale}", "vertices": V, "edges": E,
                   "iterations_per_step": ITERS, "epsilon": 0.0, "storage": "f32",
                   "l2": "inputs larger than L2 (4E = %.2f GB CSC ids per iteration)" % (4 * E / 1e9),
                   "parallelism": f"replicas x{world}", "graph_build_s": round(t_build, 2),
                   "gather_shape": tune},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "kernel": kernel, "alg_bytes_per_launch": alg,
                     "launch_ms": per_launch_ms, "peak_source": peak_kind, "iteration": iteration},
        "e2e": {"value": e2e_value, "unit": "GTEPS", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "steps": e2e_steps, "call": "pageRankGraphCSR + freePageRankStats (ctypes, no Python copies)",
                "ms_per_call": {"min": min(call_ms), "median": statistics.median(call_ms), "max": max(call_ms)}},
        "gpu_launches": launches,
        "clocks": clk,
    }

    if rank == 0 and world == 1 and not a.no_cpu:
        from oracle import oracle_ctypes as O
        threads = os.cpu_count() or 1
        _, _, dt1, _ = cpu_pagerank(graph, O, 1, threads)
        n = int(max(1, min(ITERS, 12.0 / max(dt1, 1e-3))))
        _, _, dt, _ = cpu_pagerank(graph, O, n, threads)
        line["cpu_baseline"] = {"value": E * n / dt / 1e9, "unit": "GTEPS", "cores": threads, "kind": "port",
                                "sample": f"{n} PageRank pull iterations over the same R-MAT-{a.scale} graph"}

    if rank == 0 and not a.no_extras:
        line["extras"] = extras(gg, graph, dg, V, E, sptr, torch, peak)

    if rank == 0:
        print(json.dumps(line), flush=True)
    if dg.h:
        dg.free()
    reps.close()


def splitmix_sources(V, deg, n, seed):
    """n distinct vertices of nonzero degree drawn from SplitMix64(seed)."""
    out, i = [], 0
    mask = (1 << 64) - 1
    while len(out) < n:
        z = (seed + (i + 1) * 0x9E3779B97F4A7C15) & mask
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & mask
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & mask
        z ^= z >> 31
        v = z % V
        if deg[v] and v not in out:
            out.append(int(v))
        i += 1
    return out


def ppr_extras(gg, torch, peak, scale=22, K=64, iters=20):
    """Batched personalised PageRank: K one-hot seed vectors (SplitMix64 from
    vertices with out-edges) over a directed R-MAT graph, one multi-vector
    pull gather per iteration; aggregate GTEPS = K*E*iters/t, roofline
    against 4E + 8V + K*V*4s bytes per iteration, L1 vs FP64 for 4 vectors;
    the CPU baseline runs the same vectors in FP32 on the host cores."""
    import numpy as np
    from oracle import oracle_ctypes as O

    g = gg.Graph.rmat(scale, 16, seed=SEED)
    V, E = g.V, g.E
    dg = gg.DeviceGraph(g, gg.MAP_IN)
    deg = g.views()["out_degree"]
    seeds = splitmix_sources(V, deg, K, SEED + 3)
    sets = [[s] for s in seeds]
    out = {"graph": f"R-MAT-{scale} directed, V={V}, E={E}", "vectors": K, "iterations": iters}
    a = g.arrays()
    o = O.Csr.from_arrays(V, E, a["out_off"], a["out_adj"], a["in_off"], a["in_adj"])
    check = [0, 1, K // 2, K - 1]
    exact = {k: O.ppr_f64_multi(o, sets[k], iters, float(np.float32(0.85))) for k in check}
    for storage, s in [("bf16", 2), ("f32", 4)]:
        for _ in range(2):
            dg.ppr(sets, iterations=iters, storage=storage, copy_out=False)
        torch.cuda.synchronize()
        reps, gms = 5, 0.0
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            _, r = dg.ppr(sets, iterations=iters, storage=storage, copy_out=False, profile=True)
            gms += r["gather_ms"] / max(r["gather_launches"], 1)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        ranks, _ = dg.ppr(sets, iterations=iters, storage=storage)
        l1 = max(float(np.abs(ranks[:, k] - exact[k]).sum()) for k in check)
        alg = 4 * E + 8 * V + K * V * 4 * s
        out[storage] = {"gteps": K * E * iters / (ms / 1e3) / 1e9, "ms_per_run": ms,
                        "gather_launch_ms": gms / reps,
                        "iteration_hbm_frac": alg / (ms / iters / 1e3) / 1e9 / peak,
                        "alg_bytes_per_iteration": alg, "l1_vs_fp64_max": l1}
    # CPU baseline: the same K vectors in FP32, [V][K] rows, OpenMP over
    # destination vertices on every host core; a bounded sample of 2 iterations
    cpu_iters = 2
    t0 = time.perf_counter()
    O.ppr_f32_batch(o, sets, cpu_iters, float(np.float32(0.85)))
    cpu_s = time.perf_counter() - t0
    out["cpu_baseline"] = {"gteps": K * E * cpu_iters / cpu_s / 1e9, "cores": os.cpu_count(), "kind": "port",
                           "sample": f"all {K} vectors, {cpu_iters} of the {iters} iterations, FP32"}
    dg.free()
    g.free()
    return out


def c1_extras(gg, torch, scale=16, peak=6660.9):
    """The CPU-runnable configuration: PageRank pull on R-MAT-16 (65,536
    vertices, 1,048,576 edges), epsilon 1e-4, at most 20 iterations, in the
    reference's formulation (start 0.15, divide by V at the end) and with
    1/N initialisation, in the gather shape the autotuner picks for the
    graph; ranks against the FP64 oracle (L1, L-inf),
    iterations against the reference's FP32 loop, GTEPS over the iterations
    run, the oracle's OpenMP loop timed beside it."""
    import numpy as np
    from oracle import oracle_ctypes as O

    g = gg.Graph.rmat(scale, 16, seed=SEED)
    V, E = g.V, g.E
    a = g.arrays()
    o = O.Csr.from_arrays(V, E, a["out_off"], a["out_adj"], a["in_off"], a["in_adj"])
    dg = gg.DeviceGraph(g, gg.MAP_IN)
    # the gather's launch shape picked by the autotuner for this graph class
    # (setup; remembered for the class, so the drop-in calls below use it too)
    tune = dg.autotune(gg.TUNE_PR, reps=3).get("pr")
    out = {"graph": f"R-MAT-{scale}, V={V}, E={E}", "epsilon": 1e-4, "max_iterations": 20, "gather_shape": tune}
    for name, one_over_n in (("reference_formulation", False), ("init_1_over_n", True)):
        # per call (wall time, results left on the device): the call as one
        # cached CUDA graph launch, and as stream launches
        timed = {}
        for as_graph in (True, False):
            for _ in range(3):
                dg.pagerank("pull", iterations=20, epsilon=1e-4, init_one_over_n=one_over_n, copy_out=False,
                            cuda_graph=as_graph)
            reps = 20
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(reps):
                _, r = dg.pagerank("pull", iterations=20, epsilon=1e-4, init_one_over_n=one_over_n,
                                   copy_out=False, cuda_graph=as_graph)
            timed[as_graph] = (time.perf_counter() - t0) * 1e3 / reps
        ms = timed[True]
        ranks, r = dg.pagerank("pull", iterations=20, epsilon=1e-4, init_one_over_n=one_over_n)
        ref, info = O.pagerank(o, 0, 20, 1e-4, init_one_over_n=one_over_n)
        ex = O.pagerank_f64(o, info["executed"], init_one_over_n=one_over_n)
        t0 = time.perf_counter()
        O.pagerank(o, 0, 20, 1e-4, init_one_over_n=one_over_n, nthreads=os.cpu_count() or 1)
        cpu_ms = (time.perf_counter() - t0) * 1e3
        alg = pr_bytes(V, E, 4) * info["executed"]
        out[name] = {"iterations": r["iterations"], "iterations_reference_loop": info["iterations"],
                     "iterations_executed": info["executed"], "ms_per_call": ms,
                     "gteps": E * (info["executed"]) / (ms / 1e3) / 1e9,
                     "roofline": {"alg_bytes_per_call": alg, "achieved_gbs": alg / (ms / 1e3) / 1e9,
                                  "frac": alg / (ms / 1e3) / 1e9 / peak,
                                  "note": "R-MAT-16's 5.8 MB per iteration stays in L2; the call is launch-bound"},
                     "ms_per_call_stream_launches": timed[False],
                     "gteps_stream_launches": E * (info["executed"]) / (timed[False] / 1e3) / 1e9,
                     "l1_vs_fp64": float(np.abs(ranks - ex).sum()), "linf_vs_fp64": float(np.abs(ranks - ex).max()),
                     "l1_reference_fp32_loop_vs_fp64": float(np.abs(ref - ex).sum()),
                     "cpu_gteps": E * info["executed"] / (cpu_ms / 1e3) / 1e9}
    dg.free()
    # end to end through the drop-in entry point on host arrays (upload,
    # 20 iterations at epsilon 1e-4, ranks back), as a C caller makes it
    import ctypes as C
    gg.set_gpu_options(storage="f32", device=0, keep_resident=False, verbose=False)
    args = gg.default_arguments(iterations=20, epsilon=1e-4)
    L = gg.lib()
    for _ in range(3):
        L.freePageRankStats(L.pageRankGraphCSR(C.byref(args), g.ptr))
    reps = 20
    t0 = time.perf_counter()
    for _ in range(reps):
        st = L.pageRankGraphCSR(C.byref(args), g.ptr)
        if not st:
            raise gg.GgError("pageRankGraphCSR failed")
        its = st.contents.iterations
        L.freePageRankStats(st)
    e2e_ms = (time.perf_counter() - t0) * 1e3 / reps
    executed = out["reference_formulation"]["iterations_executed"]
    out["e2e"] = {"ms_per_call": e2e_ms, "gteps": E * executed / (e2e_ms / 1e3) / 1e9, "iterations": its,
                  "h2d_bytes_per_call": 4 * V + 4 + 4 * E + 4 * V, "d2h_bytes_per_call": 4 * V,
                  "call": "pageRankGraphCSR + freePageRankStats"}
    g.free()
    return out


def splitmix_unit(seed):
    """A uniform double in [0, 1) from one SplitMix64 output (53 bits)."""
    mask = (1 << 64) - 1
    z = (seed + 0x9E3779B97F4A7C15) & mask
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & mask
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & mask
    z ^= z >> 31
    return (z >> 11) / float(1 << 53)


def batch_extras(gg, torch, peak, n=4096, iters=20):
    """Many small graphs in one run: n R-MAT graphs, graph i of scale
    round(10 + 7u) with u uniform from SplitMix64(seed+4+i) (V = 2^scale,
    log-uniform between 2^10 and 2^17), edge factor 8, R-MAT seed seed+4+i.
    The many-graphs kernel ranks all of them, every iteration, in one launch
    (one CTA per graph, largest first; graphs up to the bin threshold keep
    their contributions in shared memory), in the configuration the
    autotuner picks for this batch and in the default one; the union pull
    (20 x 2 launches over the block-diagonal union, as one CUDA graph) is
    timed beside it.  Roofline: the algorithm's per-iteration bytes summed
    over the graphs.  Parity: the smallest, a middle and the largest graph
    against the FP64 oracle; CPU baseline: the oracle's OpenMP pull on 64
    graphs spread over the size range."""
    import numpy as np
    from oracle import oracle_ctypes as O

    scales = [int(round(10 + 7 * splitmix_unit(SEED + 4 + i))) for i in range(n)]
    t0 = time.perf_counter()
    g, voff = gg.Graph.rmat_batch(scales, edge_factor=8, seed0=SEED + 4)
    build_s = time.perf_counter() - t0
    V, E = g.V, g.E
    dg = gg.DeviceGraph(g, gg.MAP_IN)

    def timed(**kw):
        for _ in range(2):
            dg.pagerank_batch(voff, iterations=iters, epsilon=0.0, copy_out=False, **kw)
        torch.cuda.synchronize()
        reps = 5
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            _, r = dg.pagerank_batch(voff, iterations=iters, epsilon=0.0, copy_out=False, **kw)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps, r

    out = {"graphs": n, "vertices": V, "edges": E, "iterations": iters, "build_s": round(build_s, 1)}
    alg = pr_bytes(V, E, 4)
    runs = {}
    dg.batch_config(7, 16, 4096, 2, strategy=1)
    ms, r = timed()
    runs["many_graphs_kernel_default_shape"] = {
        "ms_per_run": ms, "gteps": E * iters / (ms / 1e3) / 1e9,
        "iteration_hbm_frac": alg / (ms / iters / 1e3) / 1e9 / peak, "launches": r["launches"],
        "shape": dg.tuned(gg.TUNE_BATCH)}
    t0 = time.perf_counter()
    tune = dg.autotune(gg.TUNE_BATCH, reps=2, vertex_off=voff)["batch"]
    tune_s = time.perf_counter() - t0
    ms, r = timed()
    runs["many_graphs_kernel"] = {"ms_per_run": ms, "gteps": E * iters / (ms / 1e3) / 1e9,
                                  "iteration_hbm_frac": alg / (ms / iters / 1e3) / 1e9 / peak,
                                  "launches": r["launches"], "shape": dg.tuned(gg.TUNE_BATCH),
                                  "autotune": tune, "autotune_s": round(tune_s, 1)}
    ms, r = timed(union=True, cuda_graph=True)
    runs["union_pull_cuda_graph"] = {"ms_per_run": ms, "gteps": E * iters / (ms / 1e3) / 1e9,
                                     "iteration_hbm_frac": alg / (ms / iters / 1e3) / 1e9 / peak,
                                     "launches": r["launches"]}
    out.update(runs)
    ranks, _ = dg.pagerank_batch(voff, iterations=iters, epsilon=0.0)
    dg.free()
    g.free()
    # parity on the smallest, a middle and the largest graph
    order = np.argsort(scales, kind="stable")
    worst = 0.0
    for i in (int(order[0]), int(order[n // 2]), int(order[-1])):
        o = O.rmat_csr(scales[i], 8, seed=SEED + 4 + i)
        ex = O.pagerank_f64(o, iters)
        part = ranks[voff[i]:voff[i + 1]]
        worst = max(worst, float(np.abs(part - ex).sum() / np.abs(ex).sum()))
    out["l1_relative_vs_fp64_max"] = worst
    # CPU baseline: 64 graphs spread over the sizes, the oracle's OpenMP pull
    threads = os.cpu_count() or 1
    cpu_e, cpu_s = 0, 0.0
    for i in order[:: max(1, n // 64)][:64]:
        o = O.rmat_csr(scales[int(i)], 8, seed=SEED + 4 + int(i))
        t0 = time.perf_counter()
        O.pagerank(o, 0, iters, 0.0, nthreads=threads)
        cpu_s += time.perf_counter() - t0
        cpu_e += o.E * iters
    out["cpu_baseline"] = {"gteps": cpu_e / cpu_s / 1e9, "cores": threads, "kind": "port",
                           "sample": "64 of the graphs, every 64th by size, 20 iterations each"}
    return out


def serving_extras(gg, scale=23, n=1500, rate=150.0):
    """The query server under Poisson arrivals (seed+5): 70% personalised
    PageRank from 1-32 random seeds, 30% BFS from a random vertex with
    out-edges, on a directed R-MAT graph with CSR and CSC resident.  Reports
    latency percentiles (server clock, submit to result in device memory),
    throughput, PPR batch sizes, and checks sampled queries: PPR bit-identical
    alone and within L1 1e-6 of FP64, BFS distances exact.  The CPU baseline
    is the per-query time of the same queries on the host cores, and the
    query rate that implies for this mix."""
    import threading
    import numpy as np
    from oracle import oracle_ctypes as O

    g = gg.Graph.rmat(scale, 16, seed=SEED)
    V = g.V
    dg = gg.DeviceGraph(g, gg.MAP_IN | gg.MAP_OUT)
    rng = np.random.default_rng(SEED + 5)
    deg = g.views()["out_degree"]
    nz = np.flatnonzero(deg)
    qs = []
    for _ in range(n):
        if rng.random() < 0.7:
            qs.append(("ppr", rng.integers(0, V, int(rng.integers(1, 33))).astype(np.uint32)))
        else:
            qs.append(("bfs", int(nz[rng.integers(0, len(nz))])))
    gaps = rng.exponential(1.0 / rate, n)
    sample = set(range(0, n, max(1, n // 48)))  # every 31st query of 1500: 49 sampled
    srv = gg.Server(dg, max_ppr_batch=64, ppr_iterations=20, ppr_storage="f32")
    srv.take(srv.submit_ppr([0]))      # warm-up: work buffers, tiles
    srv.take(srv.submit_bfs(int(nz[0])))
    tickets = [None] * n
    ready = threading.Semaphore(0)

    def producer():
        t0 = time.perf_counter()
        due = t0
        for i, (kind, arg) in enumerate(qs):
            due += gaps[i]
            d = due - time.perf_counter()
            if d > 0:
                time.sleep(d)
            tickets[i] = srv.submit_ppr(arg) if kind == "ppr" else srv.submit_bfs(arg)
            ready.release()

    th = threading.Thread(target=producer)
    th.start()
    infos, kept = [], {}
    for i in range(n):
        ready.acquire()
        res, info = srv.take(tickets[i], copy_out=i in sample)
        infos.append(info)
        if i in sample:
            kept[i] = res
    th.join()
    # the sampled queries again, each alone
    alone_ok, acc_ok = True, True
    a = g.arrays()
    o = O.Csr.from_arrays(V, g.E, a["out_off"], a["out_adj"], a["in_off"], a["in_adj"])
    l1_checked, l1_max = 0, 0.0
    for i in sorted(sample):
        kind, arg = qs[i]
        res, _ = srv.take(srv.submit_ppr(arg) if kind == "ppr" else srv.submit_bfs(arg))
        if kind == "ppr":
            alone_ok &= bool(np.array_equal(res, kept[i]))
            l1 = float(np.abs(kept[i] - O.ppr_f64_multi(o, arg, 20, float(np.float32(0.85)))).sum())
            l1_max = max(l1_max, l1)
            acc_ok &= l1 <= 1e-6
            l1_checked += 1
        else:
            alone_ok &= bool(np.array_equal(res[1], kept[i][1]))
            _, rd, _ = O.bfs(o, 2, arg)
            acc_ok &= bool(np.array_equal(kept[i][1], rd))
    srv.stop()
    dg.free()
    g.free()
    # CPU baseline: three sampled PPR queries (FP32, 20 iterations) and three
    # sampled BFS queries, each run alone on every host core
    cpu = {"ppr": [], "bfs": []}
    for i in sorted(sample):
        kind, arg = qs[i]
        if len(cpu[kind]) >= 3:
            continue
        t0 = time.perf_counter()
        if kind == "ppr":
            O.ppr_f32_batch(o, [list(arg)], 20, float(np.float32(0.85)))
        else:
            O.bfs(o, 2, arg, nthreads=os.cpu_count())
        cpu[kind].append((time.perf_counter() - t0) * 1e3)
    lat = np.array([(x["done_s"] - x["submit_s"]) * 1e3 for x in infos])
    kinds = np.array([x["kind"] for x in infos])
    span = max(x["done_s"] for x in infos) - min(x["submit_s"] for x in infos)
    out = {"graph": f"R-MAT-{scale} directed, V={V}", "queries": n, "offered_qps": rate,
           "achieved_qps": n / span, "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
           "ppr_batch_mean": float(np.mean([x["batch_size"] for x in infos if x["kind"] == 0])),
           "alone_equals_mixed": alone_ok, "sampled_results_match_oracle": acc_ok,
           "sampled": len(sample), "ppr_checked_vs_fp64": l1_checked, "ppr_l1_vs_fp64_max": l1_max,
           "all_ok": all(x["status"] == 0 for x in infos)}
    cp, cb = statistics.mean(cpu["ppr"] or [0.0]), statistics.mean(cpu["bfs"] or [0.0])
    out["cpu_baseline"] = {"ppr_ms_per_query": cp, "bfs_ms_per_query": cb,
                           "qps_capacity": 1e3 / (0.7 * cp + 0.3 * cb) if cp + cb > 0 else None,
                           "cores": os.cpu_count(), "kind": "port",
                           "sample": "3 sampled PPR and 3 sampled BFS queries, one at a time on all host cores"}
    for k, name in ((0, "ppr"), (1, "bfs")):
        sel = lat[kinds == k]
        if len(sel):
            out[f"{name}_p50_ms"] = float(np.percentile(sel, 50))
            out[f"{name}_p99_ms"] = float(np.percentile(sel, 99))
    return out


def bfs_extras(gg, torch, peak, scale=22):
    """BFS direction-optimising on an undirected R-MAT graph (each generated
    edge inserted both ways), 64 sources of nonzero degree; TEPS by the
    Graph500 convention (sum of the reached vertices' degrees / 2 per search,
    over the host wall time of the search call, results left on the device),
    harmonic mean over sources."""
    import numpy as np
    from oracle import oracle_ctypes as O

    g = gg.Graph.rmat(scale, 16, seed=SEED, symmetric=True)
    V, E = g.V, g.E
    dg = gg.DeviceGraph(g, gg.MAP_IN | gg.MAP_OUT)
    deg = g.views()["out_degree"]
    srcs = splitmix_sources(V, deg, 64, SEED + 1)
    for s in srcs[:3]:
        dg.bfs(s, "do")
    teps, ms_all, bytes_all, bu = [], [], [], 0
    for s in srcs:
        # the search itself (Graph500 timing: no copy of the tree to the host)
        t0 = time.perf_counter()
        _, _, r = dg.bfs(s, "do", copy_out=False)
        dt = time.perf_counter() - t0
        _, dist, _ = dg.bfs(s, "do", copy_out=True)
        reached = (dist > 0) | (np.arange(V) == s)
        edges = float(deg[reached].astype(np.int64).sum()) / 2.0
        teps.append(edges / dt)
        ms_all.append(dt * 1e3)
        # ids + frontier/parent probes per examined edge, parent + level per
        # reached vertex, visited + next bitmaps per bottom-up step
        bytes_all.append(8.0 * r["edges_examined"] + 8.0 * int(reached.sum()) + r["bottom_up_steps"] * V / 4.0)
        bu += r["bottom_up_steps"]
    # every search against the oracle's direction-optimising BFS (the
    # reference's BFS.c:525-803 restated): levels, processed vertices and
    # edges examined bit-exact; the oracle's OpenMP run is the CPU baseline
    v = g.views()
    out_off = np.append(v["out_edges_idx"], np.uint32(E))
    in_off = np.append(v["in_edges_idx"], np.uint32(E))
    o = O.Csr.from_arrays(V, E, out_off, v["out_adj"], in_off, v["in_adj"])
    threads = os.cpu_count() or 1
    match, counts_match, cpu_teps = 0, 0, []
    for s in srcs:
        t0 = time.perf_counter()
        _, rd, info = O.bfs(o, 2, s, nthreads=threads)
        cpu_s = time.perf_counter() - t0
        _, dist, r = dg.bfs(s, "do")
        match += int(np.array_equal(dist, rd))
        counts_match += int(r["processed_nodes"] == info["processed_nodes"]
                            and r["edges_examined"] == info["edges_examined"])
        reached = (rd > 0) | (np.arange(V) == s)
        cpu_teps.append(float(deg[reached].astype(np.int64).sum()) / 2.0 / cpu_s)
    hm = len(teps) / sum(1.0 / t for t in teps)
    out = {"graph": f"R-MAT-{scale} undirected, V={V}, E={E} directed", "sources": len(srcs),
           "gteps_harmonic": hm / 1e9, "ms_mean": float(np.mean(ms_all)),
           "alg_gbs_mean": float(np.mean([b / (m / 1e3) for b, m in zip(bytes_all, ms_all)]) / 1e9),
           "hbm_frac_mean": float(np.mean([b / (m / 1e3) for b, m in zip(bytes_all, ms_all)]) / 1e9 / peak),
           "bottom_up_steps_mean": bu / len(srcs),
           "levels_match_oracle": f"{match}/{len(srcs)}",
           "processed_and_edges_examined_match_oracle": f"{counts_match}/{len(srcs)}",
           "cpu_baseline_gteps": len(cpu_teps) / sum(1.0 / t for t in cpu_teps) / 1e9, "cpu_cores": threads}
    dg.free()
    g.free()
    return out


def cc_extras(gg, torch, peak):
    """Connected components (all three algorithms) on R-MAT-22 undirected
    (the BFS graph) and R-MAT-24 directed (the PageRank graph): device time
    of one gg_cc call (CUDA events on its stream, labels left on the device),
    edges per second, labels against the oracle; the CPU baseline is the
    reference's Afforest restated with OpenMP on all host cores."""
    import numpy as np
    from oracle import oracle_ctypes as O

    out = {}
    threads = os.cpu_count() or 1
    for name, scale, sym in (("rmat22u", 22, True), ("rmat24", 24, False)):
        g = gg.Graph.rmat(scale, 16, seed=SEED, symmetric=sym)
        V, E = g.V, g.E
        dg = gg.DeviceGraph(g, gg.MAP_OUT | gg.MAP_IN)
        st = torch.cuda.current_stream()
        v = g.views()
        o = O.Csr.from_arrays(V, E, np.append(v["out_edges_idx"], np.uint32(E)), v["out_adj"],
                              np.append(v["in_edges_idx"], np.uint32(E)), v["in_adj"])
        t0 = time.perf_counter()
        cpu = O.cc_afforest(o, use_in=not sym, nthreads=threads)
        cpu_s = time.perf_counter() - t0
        gold = O.cc_min_label(o)
        res = {"V": V, "E": E, "components": int(len(np.unique(gold))),
               "cpu_afforest_ms": cpu_s * 1e3, "cpu_cores": threads,
               "cpu_matches_oracle": bool(np.array_equal(cpu, gold))}
        for alg in ("afforest", "sv", "weakly"):
            use_in = 0 if sym else 1
            for _ in range(2):
                dg.cc(alg, use_in_edges=use_in, copy_out=False, stream=st.cuda_stream)
            torch.cuda.synchronize()
            ms = []
            for _ in range(5):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(st)
                _, r = dg.cc(alg, use_in_edges=use_in, copy_out=False, stream=st.cuda_stream)
                e1.record(st)
                torch.cuda.synchronize()
                ms.append(e0.elapsed_time(e1))
            comp, r = dg.cc(alg, use_in_edges=use_in, stream=st.cuda_stream)
            t = float(np.median(ms))
            res[alg] = {"ms": t, "gedges_s": E / (t / 1e3) / 1e9, "iterations": r["iterations"],
                        "launches": r["launches"], "labels_match_oracle": bool(np.array_equal(comp, gold))}
        res["afforest_vs_cpu"] = cpu_s * 1e3 / res["afforest"]["ms"]
        out[name] = res
        dg.free()
        g.free()
    return out


def relabel_extras(gg, torch, peak, scale=24):
    """PageRank pull (FP32, hot-vertex table on) on R-MAT-24 relabelled by the
    -l modes that group vertices by out-degree (the pull gather reads the
    contributions of in-neighbours, so a vertex's value is read out-degree
    times) and by DBG-in, against the natural order: gather time per launch and
    the whole-iteration GTEPS; the relabel order and relabelled build timed
    on the GPU (gg_relabel_order + gg_graph_build_relabelled, host edge list
    in)."""
    import ctypes as C

    import numpy as np

    L = gg.lib()
    el = L.generateRMATEdgeList(scale, 16, 0.57, 0.19, 0.19, SEED, 0, SEED + 2, 0)
    V, E = int(el.contents.num_vertices), int(el.contents.num_edges)
    out = {"graph": f"R-MAT-{scale}, V={V}, E={E}"}
    st = torch.cuda.current_stream()
    try:
        for lmode, name in ((0, "natural"), (1, "out-degree"), (4, "DBG-out"), (6, "HUBSort-out"),
                            (8, "HUBCluster-out"), (5, "DBG-in")):
            label = np.empty(V, np.uint32)
            t0 = time.perf_counter()
            gg._check(L.gg_relabel_order(el, lmode, SEED, label.ctypes.data, None), "gg_relabel_order")
            t1 = time.perf_counter()
            dg = gg.DeviceGraph.__new__(gg.DeviceGraph)
            dg.h = C.c_void_p()
            gg._check(L.gg_graph_build_relabelled(el, label.ctypes.data, gg.MAP_IN, None, C.byref(dg.h)),
                      "gg_graph_build_relabelled")
            t2 = time.perf_counter()
            dg.graph = gg._Shape(V, E)
            for _ in range(2):
                dg.pagerank("pull", iterations=ITERS, epsilon=0.0, copy_out=False, stream=st.cuda_stream)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            reps, gms = 3, 0.0
            e0.record(st)
            for _ in range(reps):
                _, r = dg.pagerank("pull", iterations=ITERS, epsilon=0.0, copy_out=False, profile=True,
                                   stream=st.cuda_stream)
                gms += r["gather_ms"] / max(r["gather_launches"], 1)
            e1.record(st)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / reps
            out[name] = {"lmode": lmode, "relabel_order_ms": (t1 - t0) * 1e3, "build_ms": (t2 - t1) * 1e3,
                         "gather_launch_ms": gms / reps, "gteps": E * ITERS / (ms / 1e3) / 1e9,
                         "hot_table": r["hot_table"]}
            dg.free()
    finally:
        L.freeEdgeList(el)
    return out


def csr_radix_bytes(V, E):
    """Bytes the device CSR + CSC build moves (unweighted): the CSR's keys
    made (8E read, 8E written), per 8-bit pass a count read (8E) and a
    scatter read + write (16E), ids and offsets split out (8E read, 4E + 4V
    written); the CSC's fields swapped in place (16E), its passes over the
    dst field only, and its split.  Returns (bytes, CSR passes)."""
    b = max(1, (max(V, 2) - 1).bit_length())
    passes = (2 * b + 7) // 8
    csc_passes = (b + 7) // 8
    csr = 16 * E + 24 * E * passes + 12 * E + 4 * V
    csc = 16 * E + 24 * E * csc_passes + 12 * E + 4 * V
    return csr + csc, passes


def csr_build_extras(gg, torch, peak, scale=24, edge_factor=16):
    """CSR + CSC of the R-MAT edge list built on the GPU (stable LSD radix
    sort, gg_graph_build_device on device-resident ids; gg_graph_build from
    the host edge list, upload included) against the host build of the same
    list (graphCSRFromEdgeList, all host cores); arrays compared in full."""
    import ctypes as C

    import numpy as np

    L = gg.lib()
    el = L.generateRMATEdgeList(scale, edge_factor, 0.57, 0.19, 0.19, SEED, 0, SEED + 2, 0)
    V, E = int(el.contents.num_vertices), int(el.contents.num_edges)
    try:
        src = torch.from_numpy(np.ctypeslib.as_array(el.contents.edges_array_src, (E,)).view(np.int32)).cuda()
        dst = torch.from_numpy(np.ctypeslib.as_array(el.contents.edges_array_dest, (E,)).view(np.int32)).cuda()
        st = torch.cuda.current_stream()
        what = gg.MAP_OUT | gg.MAP_IN
        for _ in range(2):
            gg.DeviceGraph.build(src, dst, num_vertices=V, what=what, stream=st.cuda_stream).free()
        torch.cuda.synchronize()
        ms = []
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            dg = gg.DeviceGraph.build(src, dst, num_vertices=V, what=what, stream=st.cuda_stream)
            e1.record(st)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
            got = dg.download(weights=False)
            dg.free()
        del src, dst
        # from the host edge list (pageable), the upload inside: the default
        # route, then each route of gg_set_host_copy_mode
        routes = {}
        for name in ("auto", "staged", "driver", "device"):
            gg.set_host_copy_mode(name)
            h = C.c_void_p()
            t0 = time.perf_counter()
            gg._check(L.gg_graph_build(el, what, None, C.byref(h)), "gg_graph_build")
            routes[name] = (time.perf_counter() - t0) * 1e3
            L.gg_graph_unmap(h)
        gg.set_host_copy_mode("auto")
        e2e_s = routes["auto"] / 1e3
        t0 = time.perf_counter()
        host = gg.Graph(L.graphCSRFromEdgeList(el))
        host_s = time.perf_counter() - t0
        a = host.arrays()
        equal = all(np.array_equal(got[k], a[k]) for k in ("out_off", "out_adj", "in_off", "in_adj"))
        host.free()
    finally:
        L.freeEdgeList(el)
    dev_ms = float(np.median(ms))
    alg, passes = csr_radix_bytes(V, E)
    return {"graph": f"R-MAT-{scale} edge list, V={V}, E={E}", "device_ms": dev_ms,
            "device_gedges_s": E / (dev_ms / 1e3) / 1e9, "e2e_from_host_ms": e2e_s * 1e3,
            "e2e_from_host_ms_by_copy_route": routes,
            "host_build_ms": host_s * 1e3, "host_cores": os.cpu_count() or 1,
            "radix_passes_per_direction": passes, "moved_bytes": alg,
            "hbm_frac": alg / (dev_ms / 1e3) / 1e9 / peak, "arrays_equal_host_build": bool(equal)}


def spmv_extras(gg, graph, V, E, sptr, torch, peak):
    """SpMV pull over the weighted R-MAT graph, FP32 and BF16 storage of x and
    the weights (FP32 products and sums), 30 products per run; L1 / L-inf vs
    the FP64 oracle."""
    import numpy as np
    from oracle import oracle_ctypes as O

    dg = gg.DeviceGraph(graph, gg.MAP_IN | gg.MAP_IN_W)
    v = graph.views()
    out_off = np.append(v["out_edges_idx"], np.uint32(E))
    in_off = np.append(v["in_edges_idx"], np.uint32(E))
    o = O.Csr.from_arrays(V, E, out_off, v["out_adj"], in_off, v["in_adj"], v["out_w"], v["in_w"])
    out = {}
    x0 = None
    # the autotuner's gather shape for this mapping (FP32 timings; both
    # storages then run in it), as the PageRank legs do
    tune = dg.autotune(gg.TUNE_SPMV, storage="f32", reps=3, stream=sptr).get("spmv")
    for storage, s in [("f32", 4), ("bf16", 2)]:
        dg.spmv("pull", storage=storage, iterations=2, copy_out=False, stream=sptr)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        reps, kms = 5, 0.0
        for _ in range(reps):
            _, _, r = dg.spmv("pull", storage=storage, iterations=ITERS, copy_out=False, profile=True, stream=sptr)
            kms += r["spmv_ms"] / max(r["spmv_launches"], 1)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        x, y, _ = dg.spmv("pull", storage=storage, iterations=1, stream=sptr)
        if x0 is None:
            x0 = x
            exact = O.spmv_f64(o, x)
        alg = 4 * E + s * E + 4 * (V + 1) + s * V + 4 * V
        out[f"spmv_pull_{storage}"] = {
            "gteps": E * ITERS / (ms / 1e3) / 1e9, "launch_ms": kms / reps,
            "hbm_frac": alg / (kms / reps / 1e3) / 1e9 / peak,
            "l1_relative": float(np.abs(y - exact).sum() / np.abs(exact).sum()),
            "linf_relative": float(np.abs(y - exact).max() / np.abs(exact).max()),
            "gather_shape": tune}
    dg.free()
    return out


def extras(gg, graph, dg, V, E, sptr, torch, peak):
    """Side measurements on the same box: BF16 / FP16 storage GTEPS with L1
    and L-inf error vs the FP64 oracle, SpMV pull, BFS."""
    import numpy as np
    from oracle import oracle_ctypes as O

    out = pr_storage_extras(gg, graph, dg, V, E, sptr, torch, peak)
    out["c1_rmat16"] = c1_extras(gg, torch, peak=peak)
    out.update(spmv_extras(gg, graph, V, E, sptr, torch, peak))
    dg.free()
    out["bfs_do"] = bfs_extras(gg, torch, peak)
    out["ppr_batched"] = ppr_extras(gg, torch, peak)
    out["many_graphs"] = batch_extras(gg, torch, peak)
    out["serving"] = serving_extras(gg)
    out["csr_build"] = csr_build_extras(gg, torch, peak)
    out["connected_components"] = cc_extras(gg, torch, peak)
    return out


def pr_storage_extras(gg, graph, dg, V, E, sptr, torch, peak):
    """PageRank pull in FP32 and in BF16 / FP16 storage with the FP32
    correction pass, 30 iterations: GTEPS, gather roofline, L1 / L-inf vs the
    FP64 oracle."""
    import numpy as np
    from oracle import oracle_ctypes as O

    out = {}
    v = graph.views()
    out_off = np.append(v["out_edges_idx"], np.uint32(E))
    in_off = np.append(v["in_edges_idx"], np.uint32(E))
    o = O.Csr.from_arrays(V, E, out_off, v["out_adj"], in_off, v["in_adj"])
    t0 = time.perf_counter()
    exact = O.pagerank_f64(o, ITERS)
    f64_s = time.perf_counter() - t0
    for storage, s in [("f32", 4), ("bf16", 2), ("f16", 2)]:
        for _ in range(2):
            dg.pagerank("pull", storage=storage, iterations=ITERS, epsilon=0.0, copy_out=False, stream=sptr)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = 10
        e0.record()
        gms = 0.0
        for _ in range(reps):
            _, r = dg.pagerank("pull", storage=storage, iterations=ITERS, epsilon=0.0, copy_out=False,
                               profile=True, stream=sptr)
            gms += r["gather_ms"] / max(r["gather_launches"], 1)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        ranks, _ = dg.pagerank("pull", storage=storage, iterations=ITERS, epsilon=0.0, stream=sptr)
        l1 = float(np.abs(ranks - exact).sum())
        linf = float(np.abs(ranks - exact).max())
        launch_ms = gms / reps
        out[f"pr_pull_{storage}"] = {
            "gteps": E * ITERS / (ms / 1e3) / 1e9, "ms_per_run": ms, "launch_ms": launch_ms,
            "hbm_frac": pr_gather_bytes(V, E, s) / (launch_ms / 1e3) / 1e9 / peak,
            "iteration_hbm_frac": pr_bytes(V, E, s) / (ms / ITERS / 1e3) / 1e9 / peak,
            "l1_vs_fp64": l1, "linf_vs_fp64": linf, "l1_relative": l1 / float(np.abs(exact).sum())}
    out["fp64_oracle_s"] = round(f64_s, 2)
    return out


if __name__ == "__main__":
    main()
