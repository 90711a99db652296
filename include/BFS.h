#ifndef BFS_H
#define BFS_H

/*
 * Breadth-first search on CSR: the reference's public API for this path
 * (02_capi_graph/include/algorithms/capi/BFS.h:22-61), implemented on one
 * GB300 GPU.  Only the CSR members exist; the DualOrder, Grid and list
 * members, and the CAPI-only bottomUpStepGraphCSRCAPI, are not part of the
 * drop-in (the last is replaced by the GPU bottom-up kernel).
 *
 * Semantics follow the reference (BFS.c:45-81, :241-1110):
 *   - distances[v] = 0 and parents[v] = -out_degree(v) (or -1 when 0) at
 *     start, so unreached vertices keep distance 0 and a negative parent;
 *   - a source with `source > num_vertices` returns the initial stats;
 *     otherwise arguments->source is replaced by label_array[source];
 *   - direction optimisation uses alpha = 15, beta = 18 and the reference's
 *     uint32 edge accounting (mu, mf, nf);
 *   - processed_nodes counts the reached vertices, the source included (the
 *     reference adds it with `++stats->processed_nodes` inside a printf
 *     argument, BFS.c:368);
 *   - pull (pushpull 0, the FPGA variant) runs every level bottom-up and, as
 *     on the FPGA, leaves `distances` untouched.
 * Levels are deterministic; parents found top-down depend on which CAS wins
 * and are valid BFS parents, parents found bottom-up are the first in-CSC
 * neighbour in the frontier, as in the reference.
 */

#include <stdint.h>

#include "graphConfig.h"
#include "graphCSR.h"
#include "arrayQueue.h"
#include "bitmap.h"

struct BFSStats
{
    uint32_t *distances;
    int *parents;
    uint32_t *distances_DualOrder;
    int *parents_DualOrder;
    uint32_t processed_nodes;
    uint32_t num_vertices;
    uint32_t iteration;
    double time_total;
};

#ifdef __cplusplus
extern "C" {
#endif

/* BFS.h:34 / BFS.c:45-81 */
struct BFSStats *newBFSStatsGraphCSR(struct GraphCSR *graph);
/* BFS.h:39 */
void freeBFSStats(struct BFSStats *stats);

/* Dispatcher on arguments->pushpull (BFS.c:241-282): 0 pull (bottom-up
 * every level), 1 push (top-down queues), 2 direction-optimised,
 * 3 push with bitmap frontiers, 4 direction-optimised with bitmap
 * frontiers, default direction-optimised. */
struct BFSStats *breadthFirstSearchGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct BFSStats *breadthFirstSearchPullGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct BFSStats *breadthFirstSearchPushGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct BFSStats *breadthFirstSearchDirectionOptimizedGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct BFSStats *breadthFirstSearchPushBitmapGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct BFSStats *breadthFirstSearchPushDirectionOptimizedBitmapGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);

/*
 * Single frontier steps on host-side frontiers (BFS.c:688-750, :752-803,
 * :1062-1110).  Each call uploads the frontier and stats arrays, runs one GPU
 * step and writes the results back into the host structures, so a caller
 * driving its own BFS loop gets the reference's behaviour.  Top-down steps
 * return mf (sum of -parent of every newly claimed vertex, i.e. its out-degree
 * or 1); the bottom-up step returns nf (vertices discovered).
 */
uint32_t topDownStepGraphCSR(struct GraphCSR *graph, struct ArrayQueue *sharedFrontierQueue,
                             struct ArrayQueue **localFrontierQueues, struct BFSStats *stats);
uint32_t bottomUpStepGraphCSR(struct GraphCSR *graph, struct Bitmap *bitmapCurr,
                              struct Bitmap *bitmapNext, struct BFSStats *stats);
uint32_t topDownStepUsingBitmapsGraphCSR(struct GraphCSR *graph, struct ArrayQueue *sharedFrontierQueue,
                                         struct BFSStats *stats);

#ifdef __cplusplus
}
#endif

#endif
