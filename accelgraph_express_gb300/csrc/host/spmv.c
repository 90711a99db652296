/*
 * Drop-in SpMV entry points (02_capi_graph/include/algorithms/capi/SPMV.h:51-56)
 * on the GPU runtime.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "SPMV.h"
#include "gg_host.h"

struct SPMVStats *newSPMVStatsGraphCSR(struct GraphCSR *graph)
{
    /* SPMV.c:51-72 */
    struct SPMVStats *s = (struct SPMVStats *)calloc(1, sizeof(struct SPMVStats));
    if (!s) return NULL;
    const uint32_t V = graph->num_vertices;
    s->num_vertices = V;
    s->vector_output = (float *)calloc((size_t)V + 4, sizeof(float));
    s->vector_input = (float *)calloc((size_t)V + 4, sizeof(float));
    if (!s->vector_output || !s->vector_input)
    {
        freeSPMVStats(s);
        return NULL;
    }
    return s;
}

void freeSPMVStats(struct SPMVStats *s)
{
    if (!s) return;
    free(s->vector_output);
    free(s->vector_input);
    free(s);
}

static struct SPMVStats *spmv_run(struct Arguments *arguments, struct GraphCSR *graph, uint32_t mode)
{
    if (!arguments || !graph) return NULL;
    struct SPMVStats *stats = newSPMVStatsGraphCSR(graph);
    if (!stats) return NULL;
    stats->arguments = arguments;
    const double t0 = gg_seconds();
    const int pull = mode == GG_SPMV_PULL || mode == GG_SPMV_PULL_FX;
    gg_graph *g = gpu_acquire(graph, pull ? (GG_MAP_IN | GG_MAP_IN_W) : (GG_MAP_OUT | GG_MAP_OUT_W), 0);
    if (!g)
    {
        freeSPMVStats(stats);
        return NULL;
    }
    gg_spmv_params p;
    memset(&p, 0, sizeof(p));
    p.mode = mode;
    p.storage = (mode == GG_SPMV_PULL || mode == GG_SPMV_PUSH) ? gpu_options()->storage : GG_STORE_F32;
    p.iterations = arguments->iterations;
    gg_spmv_result r;
    gg_status st = gg_spmv(g, &p, NULL, stats->vector_input, stats->vector_output, &r, NULL);
    gpu_release_call(graph, g);
    if (st != GG_OK)
    {
        gpu_report("SpMV", st);
        freeSPMVStats(stats);
        return NULL;
    }
    stats->iterations = arguments->iterations;
    stats->time_total = gg_seconds() - t0;
    if (gpu_options()->verbose)
    {
        printf(" -----------------------------------------------------\n");
        printf("| %-10s | %-8s | %-15s | \n", "Iterations", "Sum", "Time (S)");
        printf("| %-10u | %-8lf | %-15f | \n", stats->iterations, r.checksum, stats->time_total);
        printf(" -----------------------------------------------------\n");
    }
    return stats;
}

struct SPMVStats *SPMVGraphCSR(struct Arguments *arguments, struct GraphCSR *graph)
{
    /* SPMV.c:599-616; other codes fall back to pull */
    uint32_t mode = arguments ? arguments->pushpull : 0;
    if (mode > 3) mode = GG_SPMV_PULL;
    return spmv_run(arguments, graph, mode);
}

struct SPMVStats *SPMVPullGraphCSR(struct Arguments *a, struct GraphCSR *g) { return spmv_run(a, g, GG_SPMV_PULL); }
struct SPMVStats *SPMVPushGraphCSR(struct Arguments *a, struct GraphCSR *g) { return spmv_run(a, g, GG_SPMV_PUSH); }
struct SPMVStats *SPMVPullFixedPointGraphCSR(struct Arguments *a, struct GraphCSR *g) { return spmv_run(a, g, GG_SPMV_PULL_FX); }
struct SPMVStats *SPMVPushFixedPointGraphCSR(struct Arguments *a, struct GraphCSR *g) { return spmv_run(a, g, GG_SPMV_PUSH_FX); }
