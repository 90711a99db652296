#ifndef GRAPHCONFIG_H
#define GRAPHCONFIG_H

/*
 * Run parameters of the CSR traversal entry points.
 *
 * Same fields, types and order as the reference's `struct Arguments`
 * (02_capi_graph/include/config/graphConfig.h:11-52), so that a caller of the
 * reference's PageRank, BFS and SpMV CSR functions compiles against this
 * header unchanged.  The hot path reads `iterations`, `epsilon`,
 * `source`, `pushpull`, `algo_numThreads` and `ker_numThreads`; the CAPI
 * configuration words (`afu_config*`, `cu_config*`) are accepted and ignored
 * on the GPU.
 *
 * Compile-time graph flags follow the reference (graphConfig.h:7-8):
 * DIRECTED 1 means every graph carries its inverse (CSC) arrays.  WEIGHTED is
 * a per-graph property here: an EdgeList whose `edges_array_weight` is NULL
 * behaves like the reference built with WEIGHTED 0 (constant weight 0.0001f
 * in SpMV, SPMV.c:804), and one with weights behaves like WEIGHTED 1.
 */

#include <stdint.h>
#include "mt19937.h"

#ifndef WEIGHTED
#define WEIGHTED 0
#endif
#ifndef DIRECTED
#define DIRECTED 1
#endif

struct Arguments
{
    int wflag;
    int xflag;
    int sflag;
    int Sflag;
    int dflag;
    uint32_t binSize;
    uint32_t verbosity;
    uint32_t iterations;
    uint32_t trials;
    double epsilon;
    int source;
    uint32_t algorithm;
    uint32_t datastructure;
    uint32_t pushpull;
    uint32_t sort;
    uint32_t lmode;
    uint32_t lmode_l2;
    uint32_t lmode_l3;
    uint32_t mmode;
    uint32_t symmetric;
    uint32_t weighted;
    uint32_t delta;
    int pre_numThreads;
    int algo_numThreads;
    int ker_numThreads;
    char *fnameb;
    char *fnamel;
    uint32_t fnameb_format;
    uint32_t convert_format;
    mt19937state mt19937var;
    uint32_t cache_size;

    /* CAPI integration words: accepted, unused on the GPU */
    uint64_t afu_config;
    uint64_t afu_config_2;
    uint64_t cu_config;
    uint64_t cu_config_2;
    uint64_t cu_config_3;
    uint64_t cu_config_4;
};

#ifdef __cplusplus
extern "C" {
#endif

/*
 * Fill `arguments` with the reference CLI's defaults
 * (02_capi_graph/src/main/accel-graph.c:288-329): iterations 20,
 * epsilon 1e-4, source 0, pushpull 0, binSize 512, CAPI words 0x01,
 * mt19937 seeded with 27491095.
 */
void argumentsSetDefaults(struct Arguments *arguments);

#ifdef __cplusplus
}
#endif

#endif
