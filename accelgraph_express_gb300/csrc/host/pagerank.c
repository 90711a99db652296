/*
 * Drop-in PageRank entry points (02_capi_graph/include/algorithms/capi/pageRank.h:69-86)
 * on the GPU runtime.  Each entry point allocates the reference's stats
 * (newPageRankStatsGraphCSR, pageRank.c:50-78), maps the graph, runs the
 * variant through gg_pagerank, copies the ranks into stats->pageRanks and
 * fills iterations / error_total / time_total like the reference's loop.
 */
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "pageRank.h"
#include "gg_host.h"

/* realRanks[v] = v, filled on a helper thread while the GPU runs: the
 * drop-in call then holds no parallel region of the host threads (on a host
 * shared with other jobs one preempted thread would stall such a region) */
struct IdentityFill
{
    uint32_t *rr;
    uint32_t V;
    pthread_t th;
    int started;
};

static void *identity_fill(void *p)
{
    struct IdentityFill *f = (struct IdentityFill *)p;
    for (uint32_t v = 0; v < f->V; v++) f->rr[v] = v;
    return NULL;
}

static void identity_join(struct IdentityFill *f)
{
    if (f->started) pthread_join(f->th, NULL);
    f->started = 0;
}

/* stats with realRanks[v] = v; pageRanks set to base_pr when fill_ranks
 * (the GPU result overwrites them otherwise).  The arrays are recycled
 * between calls (gg_host_array_take).  With `fill` the identity is written
 * by a helper thread (join it with identity_join before the stats are
 * used); otherwise the fill runs on all host threads. */
static struct PageRankStats *stats_new(struct GraphCSR *graph, int fill_ranks, struct IdentityFill *fill)
{
    struct PageRankStats *s = (struct PageRankStats *)calloc(1, sizeof(struct PageRankStats));
    if (!s) return NULL;
    const uint32_t V = graph->num_vertices;
    s->damp = Damp;
    s->base_pr = 1.0f - s->damp;
    s->num_vertices = V;
    s->realRanks = (uint32_t *)gg_host_array_take((size_t)V * sizeof(uint32_t) + 16);
    s->pageRanks = (float *)gg_host_array_take((size_t)V * sizeof(float) + 16);
    if (!s->realRanks || !s->pageRanks)
    {
        freePageRankStats(s);
        return NULL;
    }
    const float base = s->base_pr;
    float *pr = s->pageRanks;
    uint32_t *rr = s->realRanks;
    if (fill && !fill_ranks)
    {
        fill->rr = rr;
        fill->V = V;
        fill->started = pthread_create(&fill->th, NULL, identity_fill, fill) == 0;
        if (fill->started) return s;
    }
#pragma omp parallel for schedule(static)
    for (uint32_t v = 0; v < V; v++)
    {
        if (fill_ranks) pr[v] = base;
        rr[v] = v;
    }
    return s;
}

struct PageRankStats *newPageRankStatsGraphCSR(struct GraphCSR *graph) { return stats_new(graph, 1, NULL); }

void freePageRankStats(struct PageRankStats *s)
{
    if (!s) return;
    gg_host_array_give(s->realRanks, (size_t)s->num_vertices * sizeof(uint32_t) + 16);
    gg_host_array_give(s->pageRanks, (size_t)s->num_vertices * sizeof(float) + 16);
    free(s);
}

static const char *mode_name(uint32_t mode)
{
    static const char *names[] = {"Page Rank Pull", "Page Rank Push", "Page Rank Pull FP_64", "Page Rank Push FP",
                                  "Page Rank Pull Quant_32", "Page Rank Push Quant", "Page Rank Pull DD",
                                  "Page Rank Push DD", "Page Rank Pull-Push DD", "Page Rank Pull FP_32",
                                  "Page Rank Pull FP_16", "Page Rank Pull FP_8", "Page Rank Pull Quant_16",
                                  "Page Rank Pull Quant_8"};
    return mode < 14 ? names[mode] : "Page Rank";
}

static struct PageRankStats *pagerank_run(struct Arguments *arguments, struct GraphCSR *graph, uint32_t mode)
{
    if (!arguments || !graph) return NULL;
    const GraphGpuOptions *o = gpu_options();
    struct IdentityFill fill;
    memset(&fill, 0, sizeof(fill));
    struct PageRankStats *stats = stats_new(graph, 0, &fill);
    if (!stats) return NULL;
    const double t0 = gg_seconds();
    uint32_t what;
    switch (mode)
    {
    case GG_PR_PUSH: case GG_PR_PUSH_FX64: case GG_PR_PUSH_Q: what = GG_MAP_OUT; break;
    case GG_PR_DD_PULL: case GG_PR_DD_PUSH: case GG_PR_DD_PULLPUSH: what = GG_MAP_OUT | GG_MAP_IN; break;
    default: what = GG_MAP_IN; break;
    }
    gg_graph *g = gpu_acquire(graph, what, 0);
    if (!g)
    {
        identity_join(&fill);
        freePageRankStats(stats);
        return NULL;
    }
    gg_pr_params p;
    memset(&p, 0, sizeof(p));
    p.mode = mode;
    p.storage = o->storage;
    p.max_iterations = arguments->iterations;
    p.epsilon = arguments->epsilon;
    p.damp = stats->damp;
    gg_pr_result r;
    gg_status st = gg_pagerank(g, &p, stats->pageRanks, &r, NULL);
    gpu_release_call(graph, g);
    identity_join(&fill);
    if (st != GG_OK)
    {
        gpu_report(mode_name(mode), st);
        freePageRankStats(stats);
        return NULL;
    }
    stats->iterations = r.iterations;
    stats->activeVertices = r.active;
    stats->error_total = r.error_total;
    stats->time_total = gg_seconds() - t0;
    if (o->verbose)
    {
        printf(" -----------------------------------------------------\n");
        printf("| %-51s | \n", mode_name(mode));
        printf(" -----------------------------------------------------\n");
        printf("| %-10s | %-8s | %-15s | %-9s | \n", "Iterations", "PR Sum", "Error", "Time (S)");
        printf(" -----------------------------------------------------\n");
        printf("| %-10u | %-8lf | %-15.13lf | %-9f | \n", stats->iterations, r.rank_sum, stats->error_total,
               stats->time_total);
        printf(" -----------------------------------------------------\n");
    }
    return stats;
}

struct PageRankStats *pageRankGraphCSR(struct Arguments *arguments, struct GraphCSR *graph)
{
    /* pageRank.c:879-935; codes outside 0..13 fall back to pull */
    uint32_t mode = arguments ? arguments->pushpull : 0;
    if (mode > 13) mode = GG_PR_PULL;
    return pagerank_run(arguments, graph, mode);
}

struct PageRankStats *pageRankPullGraphCSR(struct Arguments *a, struct GraphCSR *g) { return pagerank_run(a, g, GG_PR_PULL); }
struct PageRankStats *pageRankPushGraphCSR(struct Arguments *a, struct GraphCSR *g) { return pagerank_run(a, g, GG_PR_PUSH); }
struct PageRankStats *pageRankPullFixedPoint64BitGraphCSR(struct Arguments *a, struct GraphCSR *g) { return pagerank_run(a, g, GG_PR_PULL_FX64); }
struct PageRankStats *pageRankPullFixedPoint32BitGraphCSR(struct Arguments *a, struct GraphCSR *g) { return pagerank_run(a, g, GG_PR_PULL_FX32); }
struct PageRankStats *pageRankPullFixedPoint16BitGraphCSR(struct Arguments *a, struct GraphCSR *g) { return pagerank_run(a, g, GG_PR_PULL_FX16); }
struct PageRankStats *pageRankPullFixedPoint8BitGraphCSR(struct Arguments *a, struct GraphCSR *g) { return pagerank_run(a, g, GG_PR_PULL_FX8); }
struct PageRankStats *pageRankPushFixedPointGraphCSR(struct Arguments *a, struct GraphCSR *g) { return pagerank_run(a, g, GG_PR_PUSH_FX64); }
struct PageRankStats *pageRankPullQuant32BitGraphCSR(struct Arguments *a, struct GraphCSR *g) { return pagerank_run(a, g, GG_PR_PULL_Q32); }
struct PageRankStats *pageRankPullQuant16BitGraphCSR(struct Arguments *a, struct GraphCSR *g) { return pagerank_run(a, g, GG_PR_PULL_Q16); }
struct PageRankStats *pageRankPullQuant8BitGraphCSR(struct Arguments *a, struct GraphCSR *g) { return pagerank_run(a, g, GG_PR_PULL_Q8); }
struct PageRankStats *pageRankPushQuantGraphCSR(struct Arguments *a, struct GraphCSR *g) { return pagerank_run(a, g, GG_PR_PUSH_Q); }
struct PageRankStats *pageRankDataDrivenPullGraphCSR(struct Arguments *a, struct GraphCSR *g) { return pagerank_run(a, g, GG_PR_DD_PULL); }
struct PageRankStats *pageRankDataDrivenPushGraphCSR(struct Arguments *a, struct GraphCSR *g) { return pagerank_run(a, g, GG_PR_DD_PUSH); }
struct PageRankStats *pageRankDataDrivenPullPushGraphCSR(struct Arguments *a, struct GraphCSR *g) { return pagerank_run(a, g, GG_PR_DD_PULLPUSH); }
