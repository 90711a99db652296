#ifndef PAGERANK_H
#define PAGERANK_H

/*
 * PageRank on CSR: the reference's public API for this path
 * (02_capi_graph/include/algorithms/capi/pageRank.h), implemented on one
 * GB300 GPU.  Only the CSR members exist here; the Grid / AdjArrayList /
 * AdjLinkedList members of the reference header belong to other data
 * structures and are not part of the drop-in.
 *
 * Semantics follow the reference (pageRank.c:50-78, :942-1109):
 * ranks start at base_pr = 1 - Damp = 0.15 (unnormalised), each iteration
 * gathers contrib[u] = rank[u]/outdeg[u] (0 when outdeg is 0, no dangling
 * redistribution) over in-edges, sets rank = 0.15 + 0.85*sum, counts
 * vertices with |delta| >= epsilon and stops when that count is 0 or after
 * `iterations`; finally rank /= num_vertices.  `stats->iterations` is the
 * index of the last iteration run when the loop broke early, else
 * `iterations`; `error_total` is the last iteration's sum |delta|/V.
 *
 * The returned stats and its arrays are owned by the caller
 * (freePageRankStats).  On a GPU failure the functions print a message to
 * stderr and return NULL; graphGpuLastError() holds the status.
 */

#include <stdint.h>

#include "graphConfig.h"
#include "graphCSR.h"

#define Damp 0.85f

struct PageRankStats
{
    float damp;
    float base_pr;
    uint32_t iterations;
    uint32_t num_vertices;
    uint32_t activeVertices;
    uint32_t *realRanks;
    float *pageRanks;
    double time_total;
    double error_total;
};

#ifdef __cplusplus
extern "C" {
#endif

/* pageRank.h:32 / pageRank.c:50-78 */
struct PageRankStats *newPageRankStatsGraphCSR(struct GraphCSR *graph);
/* pageRank.h:37 */
void freePageRankStats(struct PageRankStats *stats);

/* CAS-loop atomics of the reference (pageRank.h:44-47, pageRank.c:188-252) */
void addAtomicFixedPoint(uint64_t *num, uint64_t value);
void addAtomicFloat(float *num, float value);
void addAtomicDouble(double *num, double value);
void setAtomic(uint64_t *num, uint64_t value);

void pageRankPrint(float *pageRankArray, uint32_t num_vertices);
void swapWorkLists(uint8_t **workList1, uint8_t **workList2);
void resetWorkList(uint8_t *workList, uint32_t size);
void setWorkList(uint8_t *workList, uint32_t size);

/* Dispatcher on arguments->pushpull (pageRank.c:874-939):
 * 0 pull FP32, 1 push FP32, 2 pull fixed64, 3 push fixed64,
 * 4 pull quant32, 5 push quant, 6/7/8 data-driven pull/push/pull-push,
 * 9/10/11 pull fixed32/16/8, 12/13 pull quant16/8, default pull. */
struct PageRankStats *pageRankGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct PageRankStats *pageRankPullGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct PageRankStats *pageRankPushGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);

struct PageRankStats *pageRankPullFixedPoint64BitGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct PageRankStats *pageRankPullFixedPoint32BitGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct PageRankStats *pageRankPullFixedPoint16BitGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct PageRankStats *pageRankPullFixedPoint8BitGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct PageRankStats *pageRankPushFixedPointGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);

struct PageRankStats *pageRankPullQuant32BitGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct PageRankStats *pageRankPullQuant16BitGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct PageRankStats *pageRankPullQuant8BitGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct PageRankStats *pageRankPushQuantGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);

struct PageRankStats *pageRankDataDrivenPullGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct PageRankStats *pageRankDataDrivenPushGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct PageRankStats *pageRankDataDrivenPullPushGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);

#ifdef __cplusplus
}
#endif

#endif
