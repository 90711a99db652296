/*
 * Drop-in BFS entry points (02_capi_graph/include/algorithms/capi/BFS.h:45-61)
 * on the GPU runtime.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "BFS.h"
#include "gg_host.h"

struct BFSStats *newBFSStatsGraphCSR(struct GraphCSR *graph)
{
    /* BFS.c:45-81: distances 0, parents -out_degree (or -1) */
    struct BFSStats *s = (struct BFSStats *)calloc(1, sizeof(struct BFSStats));
    if (!s) return NULL;
    const uint32_t V = graph->num_vertices;
    s->num_vertices = V;
    s->distances = (uint32_t *)malloc((size_t)V * 4 + 16);
    s->distances_DualOrder = (uint32_t *)malloc((size_t)V * 4 + 16);
    s->parents = (int *)malloc((size_t)V * 4 + 16);
    s->parents_DualOrder = (int *)malloc((size_t)V * 4 + 16);
    if (!s->distances || !s->distances_DualOrder || !s->parents || !s->parents_DualOrder)
    {
        freeBFSStats(s);
        return NULL;
    }
#pragma omp parallel for schedule(static)
    for (uint32_t v = 0; v < V; v++)
    {
        uint32_t d = graph->vertices->out_degree[v];
        s->distances[v] = 0;
        s->parents[v] = d ? -(int)d : -1;
        s->parents_DualOrder[v] = s->parents[v];
    }
    return s;
}

void freeBFSStats(struct BFSStats *s)
{
    if (!s) return;
    free(s->distances);
    free(s->distances_DualOrder);
    free(s->parents);
    free(s->parents_DualOrder);
    free(s);
}

static struct BFSStats *bfs_run(struct Arguments *arguments, struct GraphCSR *graph, uint32_t mode)
{
    if (!arguments || !graph) return NULL;
    struct BFSStats *stats = newBFSStatsGraphCSR(graph);
    if (!stats) return NULL;
    /* BFS.c:293-301: `source > num_vertices` compares as unsigned and
     * returns the initial stats; source == num_vertices would read past
     * label_array in the reference and is rejected the same way here */
    if ((uint32_t)arguments->source >= graph->num_vertices)
        return stats;
    const uint32_t *labels = graph->sorted_edges_array ? graph->sorted_edges_array->label_array : NULL;
    arguments->source = labels ? (int)labels[arguments->source] : arguments->source;

    const double t0 = gg_seconds();
    uint32_t what = mode == GG_BFS_PULL ? GG_MAP_IN
                    : (mode == GG_BFS_PUSH || mode == GG_BFS_PUSH_BITMAP) ? GG_MAP_OUT
                                                                           : (GG_MAP_OUT | GG_MAP_IN);
    gg_graph *g = gpu_acquire(graph, what, 0);
    if (!g)
    {
        freeBFSStats(stats);
        return NULL;
    }
    gg_bfs_params p;
    memset(&p, 0, sizeof(p));
    p.mode = mode;
    p.source = (uint32_t)arguments->source;
    p.alpha = 15;
    p.beta = 18;
    gg_bfs_result r;
    gg_status st = gg_bfs(g, &p, stats->parents, stats->distances, &r, NULL);
    gpu_release_call(graph, g);
    if (st != GG_OK)
    {
        gpu_report("breadth-first search", st);
        freeBFSStats(stats);
        return NULL;
    }
    stats->processed_nodes = r.processed_nodes;
    stats->iteration = 1 + r.levels;
    stats->time_total = gg_seconds() - t0;
    if (gpu_options()->verbose)
    {
        printf(" -----------------------------------------------------\n");
        printf("| %-15s | %-15s | %-15s | \n", "Iterations", "Nodes", "Time (Seconds)");
        printf("| %-15u | %-15u | %-15f | \n", stats->iteration, stats->processed_nodes, stats->time_total);
        printf(" -----------------------------------------------------\n");
    }
    return stats;
}

struct BFSStats *breadthFirstSearchGraphCSR(struct Arguments *arguments, struct GraphCSR *graph)
{
    /* BFS.c:246-266; other codes fall to direction-optimised */
    uint32_t mode = arguments ? arguments->pushpull : GG_BFS_DO;
    if (mode > 4) mode = GG_BFS_DO;
    return bfs_run(arguments, graph, mode);
}

struct BFSStats *breadthFirstSearchPullGraphCSR(struct Arguments *a, struct GraphCSR *g) { return bfs_run(a, g, GG_BFS_PULL); }
struct BFSStats *breadthFirstSearchPushGraphCSR(struct Arguments *a, struct GraphCSR *g) { return bfs_run(a, g, GG_BFS_PUSH); }
struct BFSStats *breadthFirstSearchDirectionOptimizedGraphCSR(struct Arguments *a, struct GraphCSR *g) { return bfs_run(a, g, GG_BFS_DO); }
struct BFSStats *breadthFirstSearchPushBitmapGraphCSR(struct Arguments *a, struct GraphCSR *g) { return bfs_run(a, g, GG_BFS_PUSH_BITMAP); }
struct BFSStats *breadthFirstSearchPushDirectionOptimizedBitmapGraphCSR(struct Arguments *a, struct GraphCSR *g) { return bfs_run(a, g, GG_BFS_DO_BITMAP); }

/* ---- single steps on host frontiers (BFS.c:688-750, :752-803, :1062-1110) ---- */

uint32_t topDownStepGraphCSR(struct GraphCSR *graph, struct ArrayQueue *shared, struct ArrayQueue **locals,
                             struct BFSStats *stats)
{
    (void)locals;
    gg_graph *g = gpu_acquire(graph, GG_MAP_OUT, 1);
    if (!g) return 0;
    uint32_t n = 0, mf = 0;
    /* the claimed vertices land after the live window, as the reference's
     * flushArrayQueueToShared does; slideWindowArrayQueue exposes them */
    gg_status st = gg_bfs_step_host(g, 0, shared->queue + shared->head, shared->tail - shared->head, 0, stats->parents,
                                    stats->distances, shared->queue + shared->tail_next, NULL, &n, &mf, NULL);
    if (st != GG_OK)
    {
        gpu_report("topDownStepGraphCSR", st);
        return 0;
    }
    shared->tail_next += n;
    return mf;
}

uint32_t bottomUpStepGraphCSR(struct GraphCSR *graph, struct Bitmap *curr, struct Bitmap *next, struct BFSStats *stats)
{
    gg_graph *g = gpu_acquire(graph, GG_MAP_IN, 1);
    if (!g) return 0;
    uint32_t n = 0, nf = 0;
    gg_status st = gg_bfs_step_host(g, 1, curr->bitarray, 0, 1, stats->parents, stats->distances, NULL,
                                    next->bitarray, &n, &nf, NULL);
    if (st != GG_OK)
    {
        gpu_report("bottomUpStepGraphCSR", st);
        return 0;
    }
    return nf;
}

uint32_t topDownStepUsingBitmapsGraphCSR(struct GraphCSR *graph, struct ArrayQueue *shared, struct BFSStats *stats)
{
    gg_graph *g = gpu_acquire(graph, GG_MAP_OUT, 1);
    if (!g) return 0;
    uint32_t n = 0, mf = 0;
    gg_status st = gg_bfs_step_host(g, 0, shared->q_bitmap->bitarray, 0, 1, stats->parents, stats->distances, NULL,
                                    shared->q_bitmap_next->bitarray, &n, &mf, NULL);
    if (st != GG_OK)
    {
        gpu_report("topDownStepUsingBitmapsGraphCSR", st);
        return 0;
    }
    return mf;
}
