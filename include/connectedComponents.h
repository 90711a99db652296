#ifndef CONNECTEDCOMPONENTS_H
#define CONNECTEDCOMPONENTS_H

/*
 * Connected components on CSR: the reference's public API for this kernel
 * (02_capi_graph/include/algorithms/capi/connectedComponents.h:21-66),
 * implemented on one GB300 GPU.  Only the CSR members exist; the Grid and
 * list members are not part of the drop-in, nor is the Judy-array helper
 * addSample (the GPU samples on the device; sampleFrequentNode is kept as
 * a host function).
 *
 * connectedComponentsGraphCSR dispatches on arguments->pushpull as the
 * reference does (connectedComponents.c:337-360): 0 Shiloach-Vishkin,
 * 1 Afforest, 2 weakly connected components, anything else Afforest.
 * Every algorithm labels each vertex with the smallest vertex id of its
 * weakly connected component; `iterations` is the number of hook or
 * propagation rounds, which depends on the order of concurrent updates, as
 * in the reference; Afforest leaves it 0 as the reference's does (its table
 * reports neighbor_rounds instead).  With arguments->symmetric set
 * the Afforest final link uses the out-edges only; otherwise it also links
 * the in-edges (the reference's DIRECTED build, :538-576).  Afforest
 * advances arguments->mt19937var by its sample count (1024, or V / 2 below
 * 1024 vertices), as the reference's host sampling does (:293-302, :535);
 * the samples themselves are drawn on the device.
 *
 * Stats: components (V labels); counts and labels as the reference's
 * printCCStats leaves them (:168-200; its CSR algorithms call it on return,
 * :463, :621, :716): the component sizes sorted ascending in counts, with
 * the label of each in labels at the same index (ids that label no
 * component have count 0 and come first; ties in ascending id), so
 * labels[V-1] is the largest component's label and counts[V-1] its size.
 * printCCStats recomputes both from components and prints the five
 * largest.
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
/* :293-334: the most frequent component label among num_samples vertices
 * drawn with the caller's generator (generateRandInt % num_vertices), ties
 * to the smallest label; advances the generator by num_samples draws. */
uint32_t sampleFrequentNode(mt19937state *mt19937var, uint32_t num_vertices, uint32_t num_samples,
                            uint32_t *components);

struct CCStats *connectedComponentsGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct CCStats *connectedComponentsAfforestGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct CCStats *connectedComponentsShiloachVishkinGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct CCStats *connectedComponentsWeaklyGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
/* On the host (connectedComponents.c:722-832): every component is closed
 * under the graph's edges in both directions, and labels name a member of
 * their component.  Returns 1 (pass) or 0.  The reference's version starts
 * its flag at 1, clears it on an edge between two labels and prints PASS
 * when it ends at 0, so it reports a correct labelling as FAIL; this one
 * returns 1 for a correct labelling. */
uint32_t connectedComponentsVerifyGraphCSR(struct CCStats *stats, struct GraphCSR *graph);

#ifdef __cplusplus
}
#endif

#endif
