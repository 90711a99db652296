#ifndef CONNECTEDCOMPONENTS_H
#define CONNECTEDCOMPONENTS_H

/*
 * Connected components on CSR: the reference's public API for this kernel
 * (02_capi_graph/include/algorithms/capi/connectedComponents.h:21-66),
 * implemented on one GB300 GPU.  Only the CSR members exist; the Grid and
 * list members are not part of the drop-in, nor are the Judy-array sampling
 * helpers (addSample, sampleFrequentNode: the GPU samples on the device).
 *
 * connectedComponentsGraphCSR dispatches on arguments->pushpull as the
 * reference does (connectedComponents.c:337-360): 0 Shiloach-Vishkin,
 * 1 Afforest, 2 weakly connected components, anything else Afforest.
 * Every algorithm labels each vertex with the smallest vertex id of its
 * weakly connected component; `iterations` is the number of hook or
 * propagation rounds (Afforest: neighbor_rounds), which depends on the order
 * of concurrent updates, as in the reference.  With arguments->symmetric set
 * the Afforest final link uses the out-edges only; otherwise it also links
 * the in-edges (the reference's DIRECTED build, :538-576).
 *
 * Stats: components (V labels), counts[label] = size of that component
 * (0 for ids that are no label), labels = the vertex ids ordered by
 * descending count, ties by ascending id, so labels[0] is the largest
 * component's label (printCCStats, :168-216, prints the top five).
 */

#include <stdint.h>

#include "graphConfig.h"
#include "graphCSR.h"

struct CCStats
{
    uint32_t iterations;
    uint32_t neighbor_rounds;
    struct Arguments *arguments;
    uint32_t num_vertices;
    uint32_t *components;
    uint32_t *counts;
    uint32_t *labels;
    double time_total;
};

#ifdef __cplusplus
extern "C" {
#endif

struct CCStats *newCCStatsGraphCSR(struct GraphCSR *graph);
void freeCCStats(struct CCStats *stats);
void printCCStats(struct CCStats *stats);
void printComponents(struct CCStats *stats);

/* CPU helpers of the reference (connectedComponents.c:233-283): a
 * compare-and-swap minimum (returns 1 when it lowered *oldValue), the
 * union of two trees under the lower label, full pointer-jumping
 * compression of a label array. */
uint32_t atomicMin(uint32_t *oldValue, uint32_t newValue);
void linkNodes(uint32_t u, uint32_t v, uint32_t *components);
void compressNodes(uint32_t num_vertices, uint32_t *components);

struct CCStats *connectedComponentsGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct CCStats *connectedComponentsAfforestGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct CCStats *connectedComponentsShiloachVishkinGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct CCStats *connectedComponentsWeaklyGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
/* On the host (connectedComponents.c:722-832): every component is closed
 * under the graph's edges in both directions, and labels name a member of
 * their component.  Returns 1 (pass) or 0. */
uint32_t connectedComponentsVerifyGraphCSR(struct CCStats *stats, struct GraphCSR *graph);

#ifdef __cplusplus
}
#endif

#endif
