"""accelgraph_express_gb300: GB300-native CSR traversal (PageRank, SpMV, BFS).

The product is ``libaccelgraph_gb300.so``: the reference-compatible C entry
points (``pageRank*GraphCSR``, ``breadthFirstSearch*GraphCSR``,
``SPMV*GraphCSR``), the graph builder, and the ``gg_*`` GPU runtime, declared
in ``include/*.h``.  This module binds it with ctypes for Python callers,
tests and the benchmark; it adds no compute of its own and raises if the
library is missing or no GPU is present when a GPU call is made.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libaccelgraph_gb300.so")

_LIB = None


def build(jobs: int | None = None) -> str:
    """Compile libaccelgraph_gb300.so for sm_103a (make in csrc/)."""
    jobs = jobs or max(1, min(16, os.cpu_count() or 1))
    subprocess.check_call(["make", "-s", "-j", str(jobs), "-C", os.path.join(HERE, "csrc")])
    return LIB_PATH


# ---------------------------------------------------------------------------
# C structures (include/*.h)
# ---------------------------------------------------------------------------

class Mt19937State(C.Structure):
    _fields_ = [("mt", C.c_uint32 * 624), ("mti", C.c_int)]


class Arguments(C.Structure):
    """struct Arguments (include/graphConfig.h, reference graphConfig.h:11-52)."""
    _fields_ = [("wflag", C.c_int), ("xflag", C.c_int), ("sflag", C.c_int), ("Sflag", C.c_int),
                ("dflag", C.c_int), ("binSize", C.c_uint32), ("verbosity", C.c_uint32),
                ("iterations", C.c_uint32), ("trials", C.c_uint32), ("epsilon", C.c_double),
                ("source", C.c_int), ("algorithm", C.c_uint32), ("datastructure", C.c_uint32),
                ("pushpull", C.c_uint32), ("sort", C.c_uint32), ("lmode", C.c_uint32),
                ("lmode_l2", C.c_uint32), ("lmode_l3", C.c_uint32), ("mmode", C.c_uint32),
                ("symmetric", C.c_uint32), ("weighted", C.c_uint32), ("delta", C.c_uint32),
                ("pre_numThreads", C.c_int), ("algo_numThreads", C.c_int), ("ker_numThreads", C.c_int),
                ("fnameb", C.c_char_p), ("fnamel", C.c_char_p), ("fnameb_format", C.c_uint32),
                ("convert_format", C.c_uint32), ("mt19937var", Mt19937State), ("cache_size", C.c_uint32),
                ("afu_config", C.c_uint64), ("afu_config_2", C.c_uint64), ("cu_config", C.c_uint64),
                ("cu_config_2", C.c_uint64), ("cu_config_3", C.c_uint64), ("cu_config_4", C.c_uint64)]


class Vertex(C.Structure):
    _fields_ = [("out_degree", C.POINTER(C.c_uint32)), ("in_degree", C.POINTER(C.c_uint32)),
                ("edges_idx", C.POINTER(C.c_uint32))]


class EdgeList(C.Structure):
    _fields_ = [("num_edges", C.c_uint32), ("num_vertices", C.c_uint32), ("max_weight", C.c_float),
                ("edges_array_src", C.POINTER(C.c_uint32)), ("edges_array_dest", C.POINTER(C.c_uint32)),
                ("edges_array_weight", C.POINTER(C.c_float)), ("label_array", C.POINTER(C.c_uint32)),
                ("inverse_label_array", C.POINTER(C.c_uint32))]


class GraphCSR(C.Structure):
    _fields_ = [("num_edges", C.c_uint32), ("num_vertices", C.c_uint32), ("max_weight", C.c_float),
                ("avg_degree", C.c_uint32), ("vertices", C.POINTER(Vertex)),
                ("inverse_vertices", C.POINTER(Vertex)), ("sorted_edges_array", C.POINTER(EdgeList)),
                ("inverse_sorted_edges_array", C.POINTER(EdgeList))]


class PageRankStats(C.Structure):
    _fields_ = [("damp", C.c_float), ("base_pr", C.c_float), ("iterations", C.c_uint32),
                ("num_vertices", C.c_uint32), ("activeVertices", C.c_uint32),
                ("realRanks", C.POINTER(C.c_uint32)), ("pageRanks", C.POINTER(C.c_float)),
                ("time_total", C.c_double), ("error_total", C.c_double)]


class BFSStats(C.Structure):
    _fields_ = [("distances", C.POINTER(C.c_uint32)), ("parents", C.POINTER(C.c_int)),
                ("distances_DualOrder", C.POINTER(C.c_uint32)), ("parents_DualOrder", C.POINTER(C.c_int)),
                ("processed_nodes", C.c_uint32), ("num_vertices", C.c_uint32), ("iteration", C.c_uint32),
                ("time_total", C.c_double)]


class SPMVStats(C.Structure):
    _fields_ = [("iterations", C.c_uint32), ("arguments", C.POINTER(Arguments)),
                ("num_vertices", C.c_uint32), ("vector_output", C.POINTER(C.c_float)),
                ("vector_input", C.POINTER(C.c_float)), ("time_total", C.c_double)]


class Bitmap(C.Structure):
    _fields_ = [("size", C.c_uint32), ("numSetBits", C.c_uint32), ("bitarray", C.POINTER(C.c_uint32))]


class ArrayQueue(C.Structure):
    _fields_ = [("head", C.c_uint32), ("tail", C.c_uint32), ("tail_next", C.c_uint32), ("size", C.c_uint32),
                ("queue", C.POINTER(C.c_uint32)), ("q_bitmap", C.POINTER(Bitmap)),
                ("q_bitmap_next", C.POINTER(Bitmap))]


class CCStats(C.Structure):
    _fields_ = [("iterations", C.c_uint32), ("neighbor_rounds", C.c_uint32), ("arguments", C.c_void_p),
                ("num_vertices", C.c_uint32), ("components", C.POINTER(C.c_uint32)),
                ("counts", C.POINTER(C.c_uint32)), ("labels", C.POINTER(C.c_uint32)), ("time_total", C.c_double)]


class CcParams(C.Structure):
    _fields_ = [("algorithm", C.c_uint32), ("neighbor_rounds", C.c_uint32), ("samples", C.c_uint32),
                ("use_in_edges", C.c_uint32), ("max_iterations", C.c_uint32), ("profile", C.c_uint32),
                ("seed", C.c_uint64)]


class CcResult(C.Structure):
    _fields_ = [("iterations", C.c_uint32), ("components", C.c_uint32), ("launches", C.c_uint32),
                ("skipped_label", C.c_uint32), ("kernel_ms", C.c_float)]


CC_ALGORITHMS = {"sv": 0, "afforest": 1, "weakly": 2}


class PrParams(C.Structure):
    _fields_ = [("mode", C.c_uint32), ("storage", C.c_uint32), ("max_iterations", C.c_uint32),
                ("init_one_over_n", C.c_uint32), ("epsilon", C.c_double), ("damp", C.c_float),
                ("profile", C.c_uint32), ("flags", C.c_uint32)]


PR_CUDA_GRAPH, PR_HOT_OFF, PR_HOT_ON, PR_BATCH_UNION = 0x1, 0x2, 0x4, 0x8


def _pr_flags(cuda_graph, hot):
    f = PR_CUDA_GRAPH if cuda_graph else 0
    if hot is True:
        f |= PR_HOT_ON
    elif hot is False:
        f |= PR_HOT_OFF
    return f


class PrResult(C.Structure):
    _fields_ = [("iterations", C.c_uint32), ("active", C.c_uint32), ("error_total", C.c_double),
                ("rank_sum", C.c_double), ("gather_ms", C.c_float), ("gather_launches", C.c_uint32),
                ("launches", C.c_uint32), ("hot_table", C.c_uint32)]


class BfsParams(C.Structure):
    _fields_ = [("mode", C.c_uint32), ("source", C.c_uint32), ("alpha", C.c_uint32), ("beta", C.c_uint32),
                ("profile", C.c_uint32)]


class BfsResult(C.Structure):
    _fields_ = [("processed_nodes", C.c_uint32), ("levels", C.c_uint32), ("top_down_steps", C.c_uint32),
                ("bottom_up_steps", C.c_uint32), ("edges_examined", C.c_uint64), ("step_ms", C.c_float),
                ("launches", C.c_uint32)]


class SpmvParams(C.Structure):
    _fields_ = [("mode", C.c_uint32), ("storage", C.c_uint32), ("iterations", C.c_uint32),
                ("profile", C.c_uint32), ("flags", C.c_uint32)]


class PprParams(C.Structure):
    _fields_ = [("num_vectors", C.c_uint32), ("iterations", C.c_uint32), ("damp", C.c_float),
                ("storage", C.c_uint32), ("profile", C.c_uint32)]


class PprResult(C.Structure):
    _fields_ = [("gather_ms", C.c_float), ("gather_launches", C.c_uint32), ("launches", C.c_uint32),
                ("padded_vectors", C.c_uint32), ("persistent", C.c_uint32)]


class ServerParams(C.Structure):
    _fields_ = [("max_ppr_batch", C.c_uint32), ("ppr_iterations", C.c_uint32), ("damp", C.c_float),
                ("ppr_storage", C.c_uint32), ("mem_budget_bytes", C.c_uint64), ("bfs_workers", C.c_uint32)]


class QueryInfo(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("status", C.c_uint32), ("submit_s", C.c_double), ("start_s", C.c_double),
                ("done_s", C.c_double), ("batch_size", C.c_uint32), ("bfs_levels", C.c_uint32),
                ("bfs_reached", C.c_uint32)]


class SpmvResult(C.Structure):
    _fields_ = [("checksum", C.c_double), ("spmv_ms", C.c_float), ("spmv_launches", C.c_uint32),
                ("launches", C.c_uint32)]


class GraphGpuOptions(C.Structure):
    _fields_ = [("storage", C.c_uint32), ("device", C.c_int), ("keep_resident", C.c_uint32),
                ("verbose", C.c_uint32)]


MAP_OUT, MAP_IN, MAP_OUT_W, MAP_IN_W, MAP_ALL = 0x1, 0x2, 0x4, 0x8, 0xF
STORE = {"f32": 0, "bf16": 1, "f16": 2}
PR_MODES = {"pull": 0, "push": 1, "pull_fx64": 2, "push_fx64": 3, "pull_q32": 4, "push_q": 5, "dd_pull": 6,
            "dd_push": 7, "dd_pullpush": 8, "pull_fx32": 9, "pull_fx16": 10, "pull_fx8": 11,
            "pull_q16": 12, "pull_q8": 13}
BFS_MODES = {"pull": 0, "push": 1, "do": 2, "push_bitmap": 3, "do_bitmap": 4}
SPMV_MODES = {"pull": 0, "push": 1, "pull_fx": 2, "push_fx": 3}


class TuneParams(C.Structure):
    _fields_ = [("families", C.c_uint32), ("storage", C.c_uint32), ("reps", C.c_uint32), ("ngraphs", C.c_uint32),
                ("vertex_off", C.c_void_p)]


class TuneChoice(C.Structure):
    _fields_ = [("family", C.c_uint32), ("params", C.c_uint32 * 5), ("default_ms", C.c_float),
                ("tuned_ms", C.c_float), ("candidates", C.c_uint32)]


class TuneResult(C.Structure):
    _fields_ = [("choice", TuneChoice * 5), ("n", C.c_uint32)]


TUNE_PR, TUNE_SPMV, TUNE_BFS, TUNE_PPR, TUNE_BATCH = 0x1, 0x2, 0x4, 0x8, 0x10
TUNE_NAMES = {TUNE_PR: "pr", TUNE_SPMV: "spmv", TUNE_BFS: "bfs", TUNE_PPR: "ppr", TUNE_BATCH: "batch"}


def tune_save(path):
    _check(lib().gg_tune_save(path.encode()), "gg_tune_save")


def tune_load(path):
    _check(lib().gg_tune_load(path.encode()), "gg_tune_load")


def tune_reset():
    _check(lib().gg_tune_reset(), "gg_tune_reset")


HOST_COPY = {"auto": 0, "staged": 1, "driver": 2, "device": 3}


def set_host_copy_mode(mode):
    """How pageable host arrays are copied to the device (gg_set_host_copy_mode)."""
    lib().gg_set_host_copy_mode(HOST_COPY[mode] if isinstance(mode, str) else int(mode))


def device_cache_trim():
    """Hand the library's cached device blocks back to CUDA."""
    lib().gg_device_cache_trim()


def device_cache_bytes():
    return int(lib().gg_device_cache_bytes())


class GgError(RuntimeError):
    pass


def lib() -> C.CDLL:
    """The product library.  Raises if it has not been built."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise GgError(f"{LIB_PATH} is missing: run accelgraph_express_gb300.build() first")
        L = C.CDLL(LIB_PATH)
        P = C.POINTER
        L.gg_last_error.restype = C.c_char_p
        L.gg_device_init.argtypes = [C.c_int]
        L.gg_graph_map.argtypes = [P(GraphCSR), C.c_uint32, C.c_void_p, P(C.c_void_p)]
        L.gg_graph_extend.argtypes = [C.c_void_p, P(GraphCSR), C.c_uint32, C.c_void_p]
        L.gg_graph_unmap.argtypes = [C.c_void_p]
        L.gg_graph_device_bytes.argtypes = [C.c_void_p]
        L.gg_graph_device_bytes.restype = C.c_size_t
        L.gg_device_cache_trim.argtypes = []
        L.gg_device_cache_trim.restype = None
        L.gg_device_cache_bytes.argtypes = []
        L.gg_device_cache_bytes.restype = C.c_size_t
        L.gg_pagerank.argtypes = [C.c_void_p, P(PrParams), C.c_void_p, P(PrResult), C.c_void_p]
        L.gg_pagerank_device_ranks.argtypes = [C.c_void_p]
        L.gg_pagerank_device_ranks.restype = C.c_void_p
        L.gg_bfs.argtypes = [C.c_void_p, P(BfsParams), C.c_void_p, C.c_void_p, P(BfsResult), C.c_void_p]
        L.gg_spmv.argtypes = [C.c_void_p, P(SpmvParams), C.c_void_p, C.c_void_p, C.c_void_p, P(SpmvResult),
                              C.c_void_p]
        L.gg_set_wait_timeout_ms.argtypes = [C.c_uint32]
        L.gg_set_barrier_limit_us.argtypes = [C.c_uint32]
        L.gg_set_host_copy_mode.argtypes = [C.c_uint32]
        L.gg_set_host_copy_mode.restype = None
        L.gg_host_copy_mode.restype = C.c_uint32
        L.gg_pagerank_batch_iterations.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p]
        L.gg_autotune.argtypes = [C.c_void_p, P(TuneParams), P(TuneResult), C.c_void_p]
        L.gg_tune_save.argtypes = [C.c_char_p]
        L.gg_tune_load.argtypes = [C.c_char_p]
        L.gg_tune_get.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p]
        L.gg_pagerank_batch_strategy.argtypes = [C.c_void_p, C.c_uint32]
        L.gg_pagerank_batch_config.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32]
        L.gg_ppr.argtypes = [C.c_void_p, P(PprParams), C.c_void_p, C.c_void_p, C.c_void_p, P(PprResult), C.c_void_p]
        L.gg_ppr_device_ranks.argtypes = [C.c_void_p, P(C.c_uint32)]
        L.gg_ppr_device_ranks.restype = C.c_void_p
        L.gg_server_start.argtypes = [C.c_void_p, P(ServerParams), P(C.c_void_p)]
        L.gg_server_submit_ppr.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, P(C.c_uint64)]
        L.gg_server_submit_bfs.argtypes = [C.c_void_p, C.c_uint32, P(C.c_uint64)]
        L.gg_server_take.argtypes = [C.c_void_p, C.c_uint64, C.c_uint32, P(QueryInfo), C.c_void_p, C.c_void_p,
                                     C.c_void_p]
        L.gg_server_stop.argtypes = [C.c_void_p]
        L.gg_graph_share.argtypes = [C.c_void_p, P(C.c_void_p)]
        L.newEdgeList.argtypes = [C.c_uint32, C.c_uint32, C.c_int]
        L.newEdgeList.restype = P(EdgeList)
        L.freeEdgeList.argtypes = [P(EdgeList)]
        L.readEdgeListsbin.argtypes = [C.c_char_p, C.c_int]
        L.readEdgeListsbin.restype = P(EdgeList)
        L.readEdgeListsText.argtypes = [C.c_char_p, C.c_int]
        L.readEdgeListsText.restype = P(EdgeList)
        L.generateRMATEdgeList.argtypes = [C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double,
                                           C.c_uint64, C.c_int, C.c_uint64, C.c_int]
        L.generateRMATEdgeList.restype = P(EdgeList)
        L.generateRMATBatchEdgeList.argtypes = [C.c_uint32, C.c_void_p, C.c_uint32, C.c_double, C.c_double,
                                                C.c_double, C.c_uint64, C.c_void_p]
        L.generateRMATBatchEdgeList.restype = P(EdgeList)
        L.gg_pagerank_batch.argtypes = [C.c_void_p, P(PrParams), C.c_uint32, C.c_void_p, C.c_void_p, P(PrResult),
                                        C.c_void_p]
        L.graphCSRFromEdgeList.argtypes = [P(EdgeList)]
        L.graphCSRFromEdgeList.restype = P(GraphCSR)
        L.writeEdgeListsText.argtypes = [P(EdgeList), C.c_char_p]
        L.writeEdgeListsbin.argtypes = [P(EdgeList), C.c_char_p]
        L.writeGraphCSRbin.argtypes = [P(GraphCSR), C.c_char_p]
        L.readGraphCSRbin.argtypes = [C.c_char_p]
        L.readGraphCSRbin.restype = P(GraphCSR)
        L.edgeListFromGraphCSR.argtypes = [P(GraphCSR)]
        L.edgeListFromGraphCSR.restype = P(EdgeList)
        L.graphCSRFromFile.argtypes = [C.c_char_p, C.c_uint32, C.c_int]
        L.graphCSRFromFile.restype = P(GraphCSR)
        L.writeSerializedGraphDataStructure.argtypes = [P(Arguments)]
        L.graphCSRFromEdgeListDevice.argtypes = [P(EdgeList)]
        L.graphCSRFromEdgeListDevice.restype = P(GraphCSR)
        L.graphCSRFromEdgeListRelabelDevice.argtypes = [P(EdgeList), C.c_uint32, C.c_uint64]
        L.graphCSRFromEdgeListRelabelDevice.restype = P(GraphCSR)
        L.gg_relabel_order.argtypes = [P(EdgeList), C.c_uint32, C.c_uint64, C.c_void_p, C.c_void_p]
        L.gg_graph_build_relabelled.argtypes = [P(EdgeList), C.c_void_p, C.c_uint32, C.c_void_p, P(C.c_void_p)]
        L.gg_graph_build.argtypes = [P(EdgeList), C.c_uint32, C.c_void_p, P(C.c_void_p)]
        L.gg_graph_build_device.argtypes = [C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32,
                                            C.c_void_p, P(C.c_void_p)]
        L.gg_graph_download.argtypes = [C.c_void_p] + [C.c_void_p] * 6 + [P(C.c_float)]
        L.graphCSRFree.argtypes = [P(GraphCSR)]
        L.argumentsSetDefaults.argtypes = [P(Arguments)]
        for name in ["pageRankGraphCSR", "pageRankPullGraphCSR", "pageRankPushGraphCSR",
                     "pageRankPullFixedPoint64BitGraphCSR", "pageRankPullFixedPoint32BitGraphCSR",
                     "pageRankPullFixedPoint16BitGraphCSR", "pageRankPullFixedPoint8BitGraphCSR",
                     "pageRankPushFixedPointGraphCSR", "pageRankPullQuant32BitGraphCSR",
                     "pageRankPullQuant16BitGraphCSR", "pageRankPullQuant8BitGraphCSR",
                     "pageRankPushQuantGraphCSR", "pageRankDataDrivenPullGraphCSR",
                     "pageRankDataDrivenPushGraphCSR", "pageRankDataDrivenPullPushGraphCSR"]:
            getattr(L, name).argtypes = [P(Arguments), P(GraphCSR)]
            getattr(L, name).restype = P(PageRankStats)
        L.newPageRankStatsGraphCSR.argtypes = [P(GraphCSR)]
        L.newPageRankStatsGraphCSR.restype = P(PageRankStats)
        for name in ["breadthFirstSearchGraphCSR", "breadthFirstSearchPullGraphCSR",
                     "breadthFirstSearchPushGraphCSR", "breadthFirstSearchDirectionOptimizedGraphCSR",
                     "breadthFirstSearchPushBitmapGraphCSR",
                     "breadthFirstSearchPushDirectionOptimizedBitmapGraphCSR"]:
            getattr(L, name).argtypes = [P(Arguments), P(GraphCSR)]
            getattr(L, name).restype = P(BFSStats)
        for name in ["SPMVGraphCSR", "SPMVPullGraphCSR", "SPMVPushGraphCSR", "SPMVPullFixedPointGraphCSR",
                     "SPMVPushFixedPointGraphCSR"]:
            getattr(L, name).argtypes = [P(Arguments), P(GraphCSR)]
            getattr(L, name).restype = P(SPMVStats)
        for name in ["connectedComponentsGraphCSR", "connectedComponentsShiloachVishkinGraphCSR",
                     "connectedComponentsAfforestGraphCSR", "connectedComponentsWeaklyGraphCSR"]:
            getattr(L, name).argtypes = [P(Arguments), P(GraphCSR)]
            getattr(L, name).restype = P(CCStats)
        L.freeCCStats.argtypes = [P(CCStats)]
        L.newCCStatsGraphCSR.argtypes = [P(GraphCSR)]
        L.newCCStatsGraphCSR.restype = P(CCStats)
        L.compressNodes.argtypes = [C.c_uint32, C.c_void_p]
        L.linkNodes.argtypes = [C.c_uint32, C.c_uint32, C.c_void_p]
        L.connectedComponentsVerifyGraphCSR.argtypes = [P(CCStats), P(GraphCSR)]
        L.connectedComponentsVerifyGraphCSR.restype = C.c_uint32
        L.gg_cc.argtypes = [C.c_void_p, P(CcParams), C.c_void_p, P(CcResult), C.c_void_p]
        L.freePageRankStats.argtypes = [P(PageRankStats)]
        L.freeBFSStats.argtypes = [P(BFSStats)]
        L.freeSPMVStats.argtypes = [P(SPMVStats)]
        L.newBFSStatsGraphCSR.argtypes = [P(GraphCSR)]
        L.newBFSStatsGraphCSR.restype = P(BFSStats)
        L.topDownStepGraphCSR.argtypes = [P(GraphCSR), P(ArrayQueue), C.c_void_p, P(BFSStats)]
        L.topDownStepGraphCSR.restype = C.c_uint32
        L.bottomUpStepGraphCSR.argtypes = [P(GraphCSR), P(Bitmap), P(Bitmap), P(BFSStats)]
        L.bottomUpStepGraphCSR.restype = C.c_uint32
        L.topDownStepUsingBitmapsGraphCSR.argtypes = [P(GraphCSR), P(ArrayQueue), P(BFSStats)]
        L.topDownStepUsingBitmapsGraphCSR.restype = C.c_uint32
        L.newArrayQueue.argtypes = [C.c_uint32]
        L.newArrayQueue.restype = P(ArrayQueue)
        L.freeArrayQueue.argtypes = [P(ArrayQueue)]
        L.enArrayQueue.argtypes = [P(ArrayQueue), C.c_uint32]
        L.slideWindowArrayQueue.argtypes = [P(ArrayQueue)]
        L.newBitmap.argtypes = [C.c_uint32]
        L.newBitmap.restype = P(Bitmap)
        L.freeBitmap.argtypes = [P(Bitmap)]
        L.setBit.argtypes = [P(Bitmap), C.c_uint32]
        L.getNumOfSetBits.argtypes = [P(Bitmap)]
        L.getNumOfSetBits.restype = C.c_uint32
        L.graphGpuSetOptions.argtypes = [P(GraphGpuOptions)]
        L.graphGpuGetOptions.argtypes = [P(GraphGpuOptions)]
        L.graphGpuLastError.restype = C.c_int
        L.graphGpuRelease.argtypes = [P(GraphCSR)]
        _LIB = L
    return _LIB


def _check(st, what):
    if st != 0:
        msg = lib().gg_last_error().decode(errors="replace")
        raise GgError(f"{what}: status {st}: {msg}")


def device_init(device: int = 0):
    _check(lib().gg_device_init(device), "gg_device_init")


def _np(ptr, n, dtype):
    if n == 0 or not ptr:
        return np.zeros(0, dtype)
    ctype = {np.uint32: C.c_uint32, np.int32: C.c_int, np.float32: C.c_float}[dtype]
    return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ctype)), shape=(n,)).copy()


# ---------------------------------------------------------------------------
# host graphs
# ---------------------------------------------------------------------------

class Graph:
    """A GraphCSR built by the library (CSR + inverse CSR, uint32)."""

    def __init__(self, ptr):
        if not ptr:
            raise GgError("graph construction failed")
        self.ptr = ptr

    @staticmethod
    def _edge_list(src, dst, weights=None, num_vertices=None):
        """A library EdgeList holding copies of the arrays (free with freeEdgeList)."""
        src = np.ascontiguousarray(src, np.uint32)
        dst = np.ascontiguousarray(dst, np.uint32)
        E = len(src)
        V = int(num_vertices) if num_vertices is not None else (int(max(src.max(), dst.max())) + 1 if E else 0)
        L = lib()
        el = L.newEdgeList(E, V, 1 if weights is not None else 0)
        if not el:
            raise GgError("newEdgeList failed")
        if E:
            C.memmove(el.contents.edges_array_src, src.ctypes.data, E * 4)
            C.memmove(el.contents.edges_array_dest, dst.ctypes.data, E * 4)
            if weights is not None:
                w = np.ascontiguousarray(weights, np.float32)
                C.memmove(el.contents.edges_array_weight, w.ctypes.data, E * 4)
                el.contents.max_weight = float(w.max())
        el.contents.num_vertices = V
        return el

    @classmethod
    def from_edges_relabelled(cls, src, dst, weights=None, num_vertices=None, lmode=4, seed=27491095):
        """The GPU build of the edge list relabelled by -l mode `lmode`; the
        graph's label arrays hold the mapping (labels())."""
        L = lib()
        el = cls._edge_list(src, dst, weights, num_vertices)
        try:
            return cls(L.graphCSRFromEdgeListRelabelDevice(el, lmode, seed))
        finally:
            L.freeEdgeList(el)

    def labels(self):
        """(label_array, inverse_label_array): original id -> internal id and back."""
        e = self.ptr.contents.sorted_edges_array.contents
        return _np(e.label_array, self.V, np.uint32), _np(e.inverse_label_array, self.V, np.uint32)

    @classmethod
    def from_edges(cls, src, dst, weights=None, num_vertices=None, device_build=False):
        """device_build: sort on the GPU (graphCSRFromEdgeListDevice); the
        arrays are identical to the host build's."""
        L = lib()
        el = cls._edge_list(src, dst, weights, num_vertices)
        try:
            return cls((L.graphCSRFromEdgeListDevice if device_build else L.graphCSRFromEdgeList)(el))
        finally:
            L.freeEdgeList(el)

    @classmethod
    def rmat_batch(cls, scales, edge_factor=8, a=0.57, b=0.19, c=0.19, seed0=27491095 + 4):
        """The union of len(scales) R-MAT graphs, graph i drawn with seed
        seed0 + i and renumbered from vertex_off[i]; returns (graph, vertex_off)."""
        sc = np.ascontiguousarray(scales, np.uint32)
        voff = np.empty(len(sc) + 1, np.uint32)
        L = lib()
        el = L.generateRMATBatchEdgeList(len(sc), sc.ctypes.data, edge_factor, a, b, c, seed0, voff.ctypes.data)
        if not el:
            raise GgError("generateRMATBatchEdgeList failed")
        try:
            return cls(L.graphCSRFromEdgeList(el)), voff
        finally:
            L.freeEdgeList(el)

    @classmethod
    def rmat(cls, scale, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=27491095, weighted=False,
             weight_seed=27491095 + 2, symmetric=False, device_build=False):
        L = lib()
        el = L.generateRMATEdgeList(scale, edge_factor, a, b, c, seed, int(weighted), weight_seed, int(symmetric))
        if not el:
            raise GgError("generateRMATEdgeList failed")
        try:
            return cls((L.graphCSRFromEdgeListDevice if device_build else L.graphCSRFromEdgeList)(el))
        finally:
            L.freeEdgeList(el)

    @classmethod
    def from_file(cls, path, weighted=False, fmt=None):
        """fmt: the reference's -z code (0 text edge list, 1 binary edge
        list, 2 graphCSR binary); by default from the extension (.csr: 2,
        .bin / .wbin: 1, else 0)."""
        if fmt is None:
            fmt = 2 if path.endswith(".csr") else 1 if path.endswith("bin") else 0
        g = lib().graphCSRFromFile(path.encode(), fmt, int(weighted))
        if not g:
            raise GgError(f"cannot read {path}")
        return cls(g)

    def save(self, path):
        """Write the graphCSR binary file (the -c 2 format)."""
        if lib().writeGraphCSRbin(self.ptr, path.encode()) != 0:
            raise GgError(f"cannot write {path}")

    def save_edges(self, path, binary=True):
        """Write the edges in CSR order as a binary (.bin / .wbin) or text edge list."""
        L = lib()
        el = L.edgeListFromGraphCSR(self.ptr)
        try:
            if (L.writeEdgeListsbin if binary else L.writeEdgeListsText)(el, path.encode()) != 0:
                raise GgError(f"cannot write {path}")
        finally:
            L.freeEdgeList(el)

    @property
    def V(self):
        return int(self.ptr.contents.num_vertices)

    @property
    def E(self):
        return int(self.ptr.contents.num_edges)

    def arrays(self):
        """Copies of the CSR / CSC arrays: out_off (V+1), out_adj, in_off, in_adj,
        out_w, in_w (None when unweighted), out_degree, in_degree."""
        g = self.ptr.contents
        V, E = self.V, self.E
        ov, iv = g.vertices.contents, g.inverse_vertices.contents
        oe, ie = g.sorted_edges_array.contents, g.inverse_sorted_edges_array.contents
        out_off = np.append(_np(ov.edges_idx, V, np.uint32), np.uint32(E)).astype(np.uint32)
        in_off = np.append(_np(iv.edges_idx, V, np.uint32), np.uint32(E)).astype(np.uint32)
        d = dict(out_off=out_off, out_adj=_np(oe.edges_array_dest, E, np.uint32), in_off=in_off,
                 in_adj=_np(ie.edges_array_dest, E, np.uint32), out_degree=_np(ov.out_degree, V, np.uint32),
                 in_degree=_np(iv.out_degree, V, np.uint32), out_w=None, in_w=None)
        if oe.edges_array_weight:
            d["out_w"] = _np(oe.edges_array_weight, E, np.float32)
            d["in_w"] = _np(ie.edges_array_weight, E, np.float32)
        return d

    def views(self):
        """Zero-copy numpy views of the adjacency and degree arrays (valid
        while the graph lives): out_adj, in_adj, out_degree, in_degree,
        out_edges_idx, in_edges_idx, out_w, in_w."""
        g = self.ptr.contents
        V, E = self.V, self.E
        ov, iv = g.vertices.contents, g.inverse_vertices.contents
        oe, ie = g.sorted_edges_array.contents, g.inverse_sorted_edges_array.contents

        def view(p, n, ct):
            return np.ctypeslib.as_array(C.cast(p, C.POINTER(ct)), shape=(max(n, 1),))[:n]

        d = dict(out_adj=view(oe.edges_array_dest, E, C.c_uint32), in_adj=view(ie.edges_array_dest, E, C.c_uint32),
                 out_degree=view(ov.out_degree, V, C.c_uint32), in_degree=view(iv.out_degree, V, C.c_uint32),
                 out_edges_idx=view(ov.edges_idx, V, C.c_uint32), in_edges_idx=view(iv.edges_idx, V, C.c_uint32),
                 out_w=None, in_w=None)
        if oe.edges_array_weight:
            d["out_w"] = view(oe.edges_array_weight, E, C.c_float)
            d["in_w"] = view(ie.edges_array_weight, E, C.c_float)
        return d

    def free(self):
        if self.ptr:
            lib().graphGpuRelease(self.ptr)
            lib().graphCSRFree(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# device graphs (gg_runtime)
# ---------------------------------------------------------------------------

class _Shape:
    """Sizes of a graph that exists only on the device."""

    def __init__(self, V, E):
        self.V, self.E, self.ptr = V, E, None


class DeviceGraph:
    """A gg_graph mapping of a Graph (arrays resident in HBM)."""

    def __init__(self, graph: Graph, what=MAP_ALL, stream=None):
        self.graph = graph
        self.h = C.c_void_p()
        _check(lib().gg_graph_map(graph.ptr, what, stream, C.byref(self.h)), "gg_graph_map")

    @classmethod
    def build(cls, src, dst, weights=None, num_vertices=None, what=MAP_ALL, stream=None):
        """CSR/CSC built on the device from an edge list: numpy arrays
        (gg_graph_build uploads them) or CUDA tensors of 32-bit ids and FP32
        weights (gg_graph_build_device reads them in place)."""
        self = cls.__new__(cls)
        self.h = C.c_void_p()
        L = lib()
        if hasattr(src, "is_cuda") and src.is_cuda:
            E = int(src.numel())
            if num_vertices is None:
                raise GgError("num_vertices is required for device edge arrays")
            for t in (src, dst) + ((weights,) if weights is not None else ()):
                if not t.is_contiguous() or t.element_size() != 4 or t.numel() != E:
                    raise GgError("device edge arrays must be contiguous 32-bit tensors of one length")
            _check(L.gg_graph_build_device(int(num_vertices), E, src.data_ptr(), dst.data_ptr(),
                                           None if weights is None else weights.data_ptr(), what, stream,
                                           C.byref(self.h)), "gg_graph_build_device")
            self.graph = _Shape(int(num_vertices), E)
            return self
        el = Graph._edge_list(src, dst, weights, num_vertices)
        try:
            V, E = int(el.contents.num_vertices), int(el.contents.num_edges)
            _check(L.gg_graph_build(el, what, stream, C.byref(self.h)), "gg_graph_build")
        finally:
            L.freeEdgeList(el)
        self.graph = _Shape(V, E)
        return self

    def download(self, weights=True):
        """The mapping's arrays on the host, as Graph.arrays() names them
        (offsets with E appended); weights None when not mapped."""
        V, E = self.graph.V, self.graph.E
        d = dict(out_off=np.empty(V + 1, np.uint32), out_adj=np.empty(E, np.uint32),
                 in_off=np.empty(V + 1, np.uint32), in_adj=np.empty(E, np.uint32),
                 out_w=np.empty(E, np.float32) if weights else None, in_w=np.empty(E, np.float32) if weights else None)
        mw = C.c_float()

        def ptr(a):
            return None if a is None else a.ctypes.data

        _check(lib().gg_graph_download(self.h, ptr(d["out_off"]), ptr(d["out_adj"]), ptr(d["out_w"]),
                                       ptr(d["in_off"]), ptr(d["in_adj"]), ptr(d["in_w"]), C.byref(mw)),
               "gg_graph_download")
        d["out_off"][V] = E
        d["in_off"][V] = E
        d["max_weight"] = mw.value
        return d

    def extend(self, what, stream=None):
        if self.graph.ptr is None:
            raise GgError("a mapping built on the device has no host graph to extend from")
        _check(lib().gg_graph_extend(self.h, self.graph.ptr, what, stream), "gg_graph_extend")

    def device_bytes(self):
        return int(lib().gg_graph_device_bytes(self.h))

    def pagerank(self, mode="pull", storage="f32", iterations=20, epsilon=1e-4, init_one_over_n=False,
                 damp=0.85, profile=False, copy_out=True, stream=None, cuda_graph=False, hot=None):
        """hot: None = the library's choice (hot-vertex table from 1M vertices),
        True / False = force it on / off (pull FP32/BF16/FP16)."""
        p = PrParams(PR_MODES[mode] if isinstance(mode, str) else mode, STORE[storage], iterations,
                     int(init_one_over_n), epsilon, damp, int(profile), _pr_flags(cuda_graph, hot))
        r = PrResult()
        ranks = np.empty(self.graph.V, np.float32) if copy_out else None
        _check(lib().gg_pagerank(self.h, C.byref(p), None if ranks is None else ranks.ctypes.data, C.byref(r),
                                 stream), "gg_pagerank")
        return ranks, {k: getattr(r, k) for k, _ in PrResult._fields_}

    def pagerank_batch(self, vertex_off, mode="pull", storage="f32", iterations=20, epsilon=1e-4, damp=0.85,
                       profile=False, copy_out=True, stream=None, cuda_graph=False, hot=None, union=False):
        """PageRank of a union of graphs (vertex ranges vertex_off[i] ..
        vertex_off[i+1]); each vertex normalised by its own graph's size.
        FP32 pull runs the many-graphs kernel unless union=True."""
        voff = np.ascontiguousarray(vertex_off, np.uint32)
        p = PrParams(PR_MODES[mode] if isinstance(mode, str) else mode, STORE[storage], iterations, 0, epsilon,
                     damp, int(profile), _pr_flags(cuda_graph, hot) | (PR_BATCH_UNION if union else 0))
        r = PrResult()
        ranks = np.empty(self.graph.V, np.float32) if copy_out else None
        _check(lib().gg_pagerank_batch(self.h, C.byref(p), len(voff) - 1, voff.ctypes.data,
                                       None if ranks is None else ranks.ctypes.data, C.byref(r), stream),
               "gg_pagerank_batch")
        return ranks, {k: getattr(r, k) for k, _ in PrResult._fields_}

    def autotune(self, families=TUNE_PR, storage="f32", reps=3, vertex_off=None, stream=None):
        """gg_autotune: time candidate launch shapes on this mapping and keep
        the fastest; returns {family name: {params, default_ms, tuned_ms,
        candidates}}."""
        voff = None if vertex_off is None else np.ascontiguousarray(vertex_off, np.uint32)
        p = TuneParams(families, STORE[storage], reps, 0 if voff is None else len(voff) - 1,
                       None if voff is None else voff.ctypes.data)
        r = TuneResult()
        _check(lib().gg_autotune(self.h, C.byref(p), C.byref(r), stream), "gg_autotune")
        out = {}
        for i in range(r.n):
            c = r.choice[i]
            out[TUNE_NAMES[c.family]] = {"params": list(c.params), "default_ms": c.default_ms,
                                         "tuned_ms": c.tuned_ms, "candidates": c.candidates}
        return out

    def tuned(self, family):
        """The launch shape this mapping uses now for one GG_TUNE_* family."""
        out = (C.c_uint32 * 5)()
        _check(lib().gg_tune_get(self.h, family, out), "gg_tune_get")
        return list(out)

    def batch_iterations(self, ngraphs):
        """Per-graph iteration counts of the last many-graphs run."""
        out = np.empty(ngraphs, np.uint32)
        _check(lib().gg_pagerank_batch_iterations(self.h, ngraphs, out.ctypes.data), "gg_pagerank_batch_iterations")
        return out

    def batch_config(self, ipt=7, warps=16, smem_vmax=4096, ctas_per_sm=2, strategy=None):
        """Shape of the many-graphs kernel; strategy 1 runs it, 2 the union
        pull, 0 picks by mean graph size (None leaves it as it is)."""
        _check(lib().gg_pagerank_batch_config(self.h, ipt, warps, smem_vmax, ctas_per_sm), "gg_pagerank_batch_config")
        if strategy is not None:
            _check(lib().gg_pagerank_batch_strategy(self.h, strategy), "gg_pagerank_batch_strategy")

    def bfs(self, source, mode="do", profile=False, copy_out=True, stream=None):
        p = BfsParams(BFS_MODES[mode] if isinstance(mode, str) else mode, source, 15, 18, int(profile))
        r = BfsResult()
        V = self.graph.V
        parents = np.empty(V, np.int32) if copy_out else None
        dist = np.empty(V, np.uint32) if copy_out else None
        _check(lib().gg_bfs(self.h, C.byref(p), None if parents is None else parents.ctypes.data,
                            None if dist is None else dist.ctypes.data, C.byref(r), stream), "gg_bfs")
        return parents, dist, {k: getattr(r, k) for k, _ in BfsResult._fields_}

    def cc(self, algorithm="afforest", use_in_edges=2, neighbor_rounds=0, samples=0, seed=27491095,
           max_iterations=0, profile=False, copy_out=True, stream=None):
        """Connected components: (labels or None, result dict); every label is
        the smallest vertex id of the vertex's weakly connected component."""
        p = CcParams(CC_ALGORITHMS[algorithm] if isinstance(algorithm, str) else algorithm, neighbor_rounds,
                     samples, use_in_edges, max_iterations, int(profile), seed)
        r = CcResult()
        comp = np.empty(self.graph.V, np.uint32) if copy_out else None
        _check(lib().gg_cc(self.h, C.byref(p), None if comp is None else comp.ctypes.data, C.byref(r), stream),
               "gg_cc")
        return comp, {k: getattr(r, k) for k, _ in CcResult._fields_}

    def spmv(self, mode="pull", storage="f32", iterations=1, x=None, profile=False, copy_out=True, stream=None,
             hot=None):
        p = SpmvParams(SPMV_MODES[mode] if isinstance(mode, str) else mode, STORE[storage], iterations,
                       int(profile), _pr_flags(False, hot))
        r = SpmvResult()
        V = self.graph.V
        xin = None if x is None else np.ascontiguousarray(x, np.float32)
        xo = np.empty(V, np.float32) if copy_out else None
        y = np.empty(V, np.float32) if copy_out else None
        _check(lib().gg_spmv(self.h, C.byref(p), None if xin is None else xin.ctypes.data,
                             None if xo is None else xo.ctypes.data, None if y is None else y.ctypes.data,
                             C.byref(r), stream), "gg_spmv")
        return xo, y, {k: getattr(r, k) for k, _ in SpmvResult._fields_}

    def ppr(self, seed_sets, iterations=20, storage="bf16", damp=0.85, profile=False, copy_out=True, stream=None):
        """Batched personalised PageRank: one rank vector per seed set (1..64
        sets).  Returns (ranks as a V x K array or None, result dict)."""
        K = len(seed_sets)
        off = np.zeros(K + 1, np.uint32)
        for k, sset in enumerate(seed_sets):
            off[k + 1] = off[k] + len(sset)
        seeds = (np.concatenate([np.asarray(x, np.uint32).ravel() for x in seed_sets]) if off[-1]
                 else np.zeros(1, np.uint32))
        seeds = np.ascontiguousarray(seeds, np.uint32)
        p = PprParams(K, iterations, damp, STORE[storage], int(profile))
        r = PprResult()
        ranks = np.empty((self.graph.V, K), np.float32) if copy_out else None
        _check(lib().gg_ppr(self.h, C.byref(p), off.ctypes.data, seeds.ctypes.data,
                            None if ranks is None else ranks.ctypes.data, C.byref(r), stream), "gg_ppr")
        return ranks, {k: getattr(r, k) for k, _ in PprResult._fields_}

    def free(self):
        if self.h:
            lib().gg_graph_unmap(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# the reference-compatible entry points
# ---------------------------------------------------------------------------

def default_arguments(**kw) -> Arguments:
    a = Arguments()
    lib().argumentsSetDefaults(C.byref(a))
    for k, v in kw.items():
        setattr(a, k, v)
    return a


def set_gpu_options(storage="f32", device=0, keep_resident=False, verbose=False):
    o = GraphGpuOptions(STORE[storage], device, int(keep_resident), int(verbose))
    lib().graphGpuSetOptions(C.byref(o))


class Server:
    """Query server over a DeviceGraph mapped with MAP_IN | MAP_OUT
    (include/gg_server.h): personalised PageRank queries in one continuous
    batch, BFS queries on several workers, results held on the device until
    taken."""

    QUERY_PPR, QUERY_BFS = 0, 1

    def __init__(self, dg, max_ppr_batch=64, ppr_iterations=20, damp=0.85, ppr_storage="f32",
                 mem_budget_bytes=None, bfs_workers=2):
        self.dg = dg
        self.V = dg.graph.V
        budget = mem_budget_bytes if mem_budget_bytes is not None else 256 * 8 * self.V
        p = ServerParams(max_ppr_batch, ppr_iterations, damp, STORE[ppr_storage], budget, bfs_workers)
        self.h = C.c_void_p()
        _check(lib().gg_server_start(dg.h, C.byref(p), C.byref(self.h)), "gg_server_start")

    def submit_ppr(self, seeds):
        s = np.ascontiguousarray(seeds, np.uint32)
        t = C.c_uint64()
        _check(lib().gg_server_submit_ppr(self.h, s.ctypes.data, len(s), C.byref(t)), "gg_server_submit_ppr")
        return t.value

    def submit_bfs(self, source):
        t = C.c_uint64()
        _check(lib().gg_server_submit_bfs(self.h, source, C.byref(t)), "gg_server_submit_bfs")
        return t.value

    def take(self, ticket, timeout_ms=60000, copy_out=True):
        """(result, info dict): PPR ranks (V floats) or BFS (parents,
        distances); None when copy_out is False."""
        info = QueryInfo()
        ppr = par = dist = None
        kind = None
        if copy_out:
            ppr = np.empty(self.V, np.float32)
            par = np.empty(self.V, np.int32)
            dist = np.empty(self.V, np.uint32)
        _check(lib().gg_server_take(self.h, ticket, timeout_ms, C.byref(info),
                                    None if ppr is None else ppr.ctypes.data,
                                    None if par is None else par.ctypes.data,
                                    None if dist is None else dist.ctypes.data), "gg_server_take")
        d = {k: getattr(info, k) for k, _ in QueryInfo._fields_}
        kind = d["kind"]
        if not copy_out:
            return None, d
        return (ppr if kind == self.QUERY_PPR else (par, dist)), d

    def stop(self):
        if self.h:
            lib().gg_server_stop(self.h)
            self.h = C.c_void_p()


def pagerank_csr(graph: Graph, args: Arguments, fn="pageRankGraphCSR"):
    """Call a pageRank*GraphCSR entry point; returns (ranks, stats dict)."""
    L = lib()
    s = getattr(L, fn)(C.byref(args), graph.ptr)
    if not s:
        raise GgError(f"{fn} failed: status {L.graphGpuLastError()}: {L.gg_last_error().decode()}")
    try:
        st = s.contents
        ranks = _np(st.pageRanks, graph.V, np.float32)
        return ranks, {"iterations": st.iterations, "error_total": st.error_total, "time_total": st.time_total,
                       "activeVertices": st.activeVertices, "damp": st.damp, "base_pr": st.base_pr,
                       "realRanks": _np(st.realRanks, graph.V, np.uint32)}
    finally:
        L.freePageRankStats(s)


def relabel_order(src, dst, num_vertices=None, lmode=4, seed=27491095):
    """label[orig] = new for -l mode `lmode`, computed on the GPU (gg_relabel_order)."""
    L = lib()
    el = Graph._edge_list(src, dst, None, num_vertices)
    try:
        V = int(el.contents.num_vertices)
        label = np.empty(V, np.uint32)
        _check(L.gg_relabel_order(el, lmode, seed, label.ctypes.data, None), "gg_relabel_order")
        return label
    finally:
        L.freeEdgeList(el)


def build_relabelled(src, dst, label, weights=None, num_vertices=None, what=MAP_ALL, stream=None):
    """DeviceGraph of the edge list with ids replaced by label[id] (a permutation)."""
    L = lib()
    el = Graph._edge_list(src, dst, weights, num_vertices)
    try:
        V, E = int(el.contents.num_vertices), int(el.contents.num_edges)
        lab = np.ascontiguousarray(label, np.uint32)
        if len(lab) != V:
            raise GgError("label array must have num_vertices entries")
        dg = DeviceGraph.__new__(DeviceGraph)
        dg.h = C.c_void_p()
        _check(L.gg_graph_build_relabelled(el, lab.ctypes.data, what, stream, C.byref(dg.h)),
               "gg_graph_build_relabelled")
        dg.graph = _Shape(V, E)
        return dg
    finally:
        L.freeEdgeList(el)


def cc_csr(graph: Graph, args: Arguments, fn="connectedComponentsGraphCSR", verify=False):
    """Call a connectedComponents*GraphCSR entry point; returns (components,
    counts, labels, stats dict[, verify result])."""
    L = lib()
    s = getattr(L, fn)(C.byref(args), graph.ptr)
    if not s:
        raise GgError(f"{fn} failed: status {L.graphGpuLastError()}: {L.gg_last_error().decode()}")
    try:
        st = s.contents
        V = graph.V
        out = (_np(st.components, V, np.uint32), _np(st.counts, V, np.uint32), _np(st.labels, V, np.uint32),
               {"iterations": st.iterations, "neighbor_rounds": st.neighbor_rounds, "time_total": st.time_total})
        if verify:
            out = out + (int(L.connectedComponentsVerifyGraphCSR(s, graph.ptr)),)
        return out
    finally:
        L.freeCCStats(s)


def bfs_csr(graph: Graph, args: Arguments, fn="breadthFirstSearchGraphCSR"):
    """Call a breadthFirstSearch*GraphCSR entry point; returns (parents, distances, stats dict)."""
    L = lib()
    s = getattr(L, fn)(C.byref(args), graph.ptr)
    if not s:
        raise GgError(f"{fn} failed: status {L.graphGpuLastError()}: {L.gg_last_error().decode()}")
    try:
        st = s.contents
        return (_np(st.parents, graph.V, np.int32), _np(st.distances, graph.V, np.uint32),
                {"processed_nodes": st.processed_nodes, "iteration": st.iteration, "time_total": st.time_total,
                 "source": args.source})
    finally:
        L.freeBFSStats(s)


def spmv_csr(graph: Graph, args: Arguments, fn="SPMVGraphCSR"):
    """Call an SPMV*GraphCSR entry point; returns (x, y, stats dict)."""
    L = lib()
    s = getattr(L, fn)(C.byref(args), graph.ptr)
    if not s:
        raise GgError(f"{fn} failed: status {L.graphGpuLastError()}: {L.gg_last_error().decode()}")
    try:
        st = s.contents
        return (_np(st.vector_input, graph.V, np.float32), _np(st.vector_output, graph.V, np.float32),
                {"iterations": st.iterations, "time_total": st.time_total})
    finally:
        L.freeSPMVStats(s)
