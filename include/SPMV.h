#ifndef SPMV_H
#define SPMV_H

/*
 * Sparse matrix-vector product on CSR: the reference's public API for this
 * path (02_capi_graph/include/algorithms/capi/SPMV.h:19-56), implemented on
 * one GB300 GPU.  Only the CSR members exist here.
 *
 * Semantics follow the reference (SPMV.c:594-1135):
 *   - x[v] = 1/out_degree(v), or 0.001 when the out-degree is 0 (:696-701);
 *   - pull: y[v] = sum over in-edges (u,v) of w(u,v)*x[u], recomputed
 *     `iterations` times with the same x (the FPGA CU overwrites y);
 *   - push: y[dst] += w*x[src] over out-edges, and y is not reset between
 *     iterations, so it accumulates (:795-820);
 *   - w is the edge weight when the graph carries weights (the reference's
 *     WEIGHTED 1 build), else the constant 0.0001f (:804).
 * `stats->vector_input` / `vector_output` hold x and y on return.
 */

#include <stdint.h>

#include "graphConfig.h"
#include "graphCSR.h"

struct SPMVStats
{
    uint32_t iterations;
    struct Arguments *arguments;
    uint32_t num_vertices;
    float *vector_output;
    float *vector_input;
    double time_total;
};

#ifdef __cplusplus
extern "C" {
#endif

/* SPMV.h:30 / SPMV.c:51-72 */
struct SPMVStats *newSPMVStatsGraphCSR(struct GraphCSR *graph);
/* SPMV.h:35 */
void freeSPMVStats(struct SPMVStats *stats);

/* Dispatcher on arguments->pushpull (SPMV.c:594-620): 0 pull FP32,
 * 1 push FP32, 2 pull fixed point, 3 push fixed point, default pull. */
struct SPMVStats *SPMVGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct SPMVStats *SPMVPullGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct SPMVStats *SPMVPushGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct SPMVStats *SPMVPullFixedPointGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct SPMVStats *SPMVPushFixedPointGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);

#ifdef __cplusplus
}
#endif

#endif
