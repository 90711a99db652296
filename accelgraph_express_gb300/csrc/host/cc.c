/*
 * Drop-in connected-components entry points
 * (02_capi_graph/include/algorithms/capi/connectedComponents.h:21-66) on the
 * GPU runtime (gg_cc).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

#include "connectedComponents.h"
#include "gg_host.h"

#define CC_SEED 27491095ull

struct CCStats *newCCStatsGraphCSR(struct GraphCSR *graph)
{
    struct CCStats *s = (struct CCStats *)calloc(1, sizeof(struct CCStats));
    if (!s) return NULL;
    const uint32_t V = graph->num_vertices;
    s->num_vertices = V;
    s->neighbor_rounds = 2;
    s->components = (uint32_t *)malloc((size_t)V * 4 + 16);
    s->counts = (uint32_t *)calloc((size_t)V + 4, 4);
    s->labels = (uint32_t *)malloc((size_t)V * 4 + 16);
    if (!s->components || !s->counts || !s->labels)
    {
        freeCCStats(s);
        return NULL;
    }
#pragma omp parallel for schedule(static)
    for (uint32_t v = 0; v < V; v++)
        s->components[v] = s->labels[v] = v;
    return s;
}

void freeCCStats(struct CCStats *s)
{
    if (!s) return;
    free(s->components);
    free(s->counts);
    free(s->labels);
    free(s);
}

uint32_t atomicMin(uint32_t *oldValue, uint32_t newValue)
{
    for (;;)
    {
        const uint32_t seen = __atomic_load_n(oldValue, __ATOMIC_RELAXED);
        if (seen <= newValue) return 0;
        if (__sync_bool_compare_and_swap(oldValue, seen, newValue)) return 1;
    }
}

void linkNodes(uint32_t u, uint32_t v, uint32_t *components)
{
    uint32_t a = __atomic_load_n(&components[u], __ATOMIC_RELAXED);
    uint32_t b = __atomic_load_n(&components[v], __ATOMIC_RELAXED);
    while (a != b)
    {
        const uint32_t hi = a > b ? a : b, lo = a > b ? b : a;
        const uint32_t parent = __atomic_load_n(&components[hi], __ATOMIC_RELAXED);
        if (parent == lo) return;
        if (parent == hi && __sync_bool_compare_and_swap(&components[hi], hi, lo)) return;
        a = __atomic_load_n(&components[__atomic_load_n(&components[hi], __ATOMIC_RELAXED)], __ATOMIC_RELAXED);
        b = __atomic_load_n(&components[lo], __ATOMIC_RELAXED);
    }
}

void compressNodes(uint32_t num_vertices, uint32_t *components)
{
#pragma omp parallel for schedule(dynamic, 2048)
    for (uint32_t n = 0; n < num_vertices; n++)
    {
        uint32_t c = components[n];
        while (c != components[c])
            c = components[c];
        components[n] = c;
    }
}

static int cmp_u32(const void *a, const void *b)
{
    const uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
    return x < y ? -1 : x > y;
}

/* connectedComponents.c:293-334: draws num_samples vertices with the
 * caller's generator (generateRandInt % num_vertices) and returns the label
 * seen most often among their components, ties to the smallest label (the
 * reference walks its sample table in ascending label order and keeps the
 * first maximum).  0 when nothing is sampled. */
uint32_t sampleFrequentNode(mt19937state *mt19937var, uint32_t num_vertices, uint32_t num_samples,
                            uint32_t *components)
{
    if (!mt19937var || !components || num_vertices == 0 || num_samples == 0) return 0;
    uint32_t *seen = (uint32_t *)malloc((size_t)num_samples * sizeof(uint32_t));
    if (!seen) return 0;
    for (uint32_t i = 0; i < num_samples; i++)
        seen[i] = components[generateRandInt(mt19937var) % num_vertices];
    qsort(seen, num_samples, sizeof(uint32_t), cmp_u32);
    uint32_t best = 0, best_count = 0;
    for (uint32_t i = 0; i < num_samples;)
    {
        uint32_t j = i;
        while (j < num_samples && seen[j] == seen[i]) j++;
        if (j - i > best_count)
        {
            best_count = j - i;
            best = seen[i];
        }
        i = j;
    }
    free(seen);
    return best;
}

/* The arrays the reference's printCCStats leaves (connectedComponents.c:
 * 168-200), which its CSR algorithms call on return (:463, :621, :716):
 * counts[label] = size of that component, then the (count, id) pairs sorted
 * by ascending count with the ids in labels, so the largest component ends
 * at index V - 1.  The reference sorts with OpenGraph's
 * radixSortEdgesByDegree (absent): restated as a stable counting sort on
 * the count, ties in ascending id.  Each call starts again from the
 * component array, so a second call gives the same arrays.  Returns the
 * number of components. */
static uint32_t fill_counts(struct CCStats *s)
{
    const uint32_t V = s->num_vertices;
    uint32_t *size = (uint32_t *)calloc((size_t)V + 1, 4);
    uint32_t *start = (uint32_t *)calloc((size_t)V + 2, 4);
    if (!size || !start)
    {
        free(size);
        free(start);
        return 0;
    }
    for (uint32_t v = 0; v < V; v++)
        if (s->components[v] < V) size[s->components[v]]++;
    uint32_t n = 0;
    for (uint32_t v = 0; v < V; v++)
    {
        n += size[v] != 0;
        start[size[v] + 1]++;
    }
    for (uint32_t k = 0; k <= V; k++) /* start[k] = ids whose count is below k */
        start[k + 1] += start[k];
    for (uint32_t v = 0; v < V; v++)
    {
        const uint32_t pos = start[size[v]]++;
        s->counts[pos] = size[v];
        s->labels[pos] = v;
    }
    free(size);
    free(start);
    return n;
}

/* the reference's table: the five largest components from the end of the
 * sorted arrays, then the component count (connectedComponents.c:201-215) */
static void print_top(const struct CCStats *s, uint32_t components)
{
    const uint32_t V = s->num_vertices;
    printf(" -----------------------------------------------------\n");
    printf("| %-21s | %-27s | \n", "Top Clusters", "Count");
    printf(" -----------------------------------------------------\n");
    for (uint32_t k = 0; k < 5 && k < V; k++)
        printf("| %-21u | %-27u | \n", s->labels[V - 1 - k], s->counts[V - 1 - k]);
    printf(" -----------------------------------------------------\n");
    printf("| %-21s | %-27u | \n", "Num Components", components);
    printf(" -----------------------------------------------------\n");
}

static struct CCStats *cc_run(struct Arguments *arguments, struct GraphCSR *graph, uint32_t algorithm)
{
    if (!arguments || !graph) return NULL;
    struct CCStats *stats = newCCStatsGraphCSR(graph);
    if (!stats) return NULL;
    stats->arguments = arguments;
    const uint32_t V = graph->num_vertices;
    if (V == 0) return stats;
    const double t0 = gg_seconds();
    const int symmetric = arguments->symmetric != 0;
    const uint32_t what = GG_MAP_OUT | ((algorithm == GG_CC_AFFOREST && !symmetric) ? GG_MAP_IN : 0u);
    gg_graph *g = gpu_acquire(graph, what, 0);
    if (!g)
    {
        freeCCStats(stats);
        return NULL;
    }
    gg_cc_params p;
    memset(&p, 0, sizeof(p));
    p.algorithm = algorithm;
    p.neighbor_rounds = stats->neighbor_rounds;
    /* connectedComponents.c:475-479: 1024 samples, V / 2 on small graphs */
    const uint32_t samples = V < 1024 ? V / 2 : 1024;
    p.samples = samples ? samples : 1;
    p.use_in_edges = symmetric ? 0 : 1;
    p.seed = CC_SEED;
    gg_cc_result r;
    gg_status st = gg_cc(g, &p, stats->components, &r, NULL);
    gpu_release_call(graph, g);
    if (st != GG_OK)
    {
        gpu_report("connected components", st);
        freeCCStats(stats);
        return NULL;
    }
    /* the reference's Afforest draws its samples from the caller's
     * generator (sampleFrequentNode, :293-302, called at :535); the device
     * draws its own, and the caller's generator advances by the same count */
    if (algorithm == GG_CC_AFFOREST)
        for (uint32_t i = 0; i < samples; i++)
            generateRandInt(&arguments->mt19937var);
    /* the reference's Afforest never counts iterations (:470-626): its
     * stats keep the constructor's 0 and its table shows neighbor_rounds */
    stats->iterations = algorithm == GG_CC_AFFOREST ? 0u : r.iterations;
    stats->time_total = gg_seconds() - t0;
    const uint32_t ncomp = fill_counts(stats);
    if (gpu_options()->verbose)
    {
        static const char *names[] = {"Shiloach-Vishkin", "Afforest", "Weakly"};
        printf(" -----------------------------------------------------\n");
        printf("| %-51s | \n", names[algorithm]);
        printf(" -----------------------------------------------------\n");
        printf("| %-15s | %-15s | %-15s | \n", "Iterations", "Components", "Time (S)");
        printf(" -----------------------------------------------------\n");
        printf("| %-15u | %-15u | %-15f | \n",
               algorithm == GG_CC_AFFOREST ? stats->neighbor_rounds : stats->iterations, r.components,
               stats->time_total);
        printf(" -----------------------------------------------------\n");
        print_top(stats, ncomp);
    }
    return stats;
}

struct CCStats *connectedComponentsGraphCSR(struct Arguments *arguments, struct GraphCSR *graph)
{
    if (!arguments) return NULL;
    switch (arguments->pushpull)
    {
    case 0: return connectedComponentsShiloachVishkinGraphCSR(arguments, graph);
    case 2: return connectedComponentsWeaklyGraphCSR(arguments, graph);
    default: return connectedComponentsAfforestGraphCSR(arguments, graph);
    }
}

struct CCStats *connectedComponentsShiloachVishkinGraphCSR(struct Arguments *arguments, struct GraphCSR *graph)
{
    return cc_run(arguments, graph, GG_CC_SHILOACH_VISHKIN);
}

struct CCStats *connectedComponentsAfforestGraphCSR(struct Arguments *arguments, struct GraphCSR *graph)
{
    return cc_run(arguments, graph, GG_CC_AFFOREST);
}

struct CCStats *connectedComponentsWeaklyGraphCSR(struct Arguments *arguments, struct GraphCSR *graph)
{
    return cc_run(arguments, graph, GG_CC_WEAKLY);
}

void printCCStats(struct CCStats *stats)
{
    if (!stats) return;
    print_top(stats, fill_counts(stats));
}

void printComponents(struct CCStats *stats)
{
    if (!stats) return;
    for (uint32_t i = 0; i < stats->num_vertices; i++)
        printf("v : %u comp : %u \n", i, stats->components[i]);
}

static uint32_t uf_root(uint32_t *p, uint32_t x)
{
    while (p[x] != x)
    {
        p[x] = p[p[x]];
        x = p[x];
    }
    return x;
}

uint32_t connectedComponentsVerifyGraphCSR(struct CCStats *stats, struct GraphCSR *graph)
{
    if (!stats || !graph || stats->num_vertices != graph->num_vertices) return 0;
    const uint32_t V = graph->num_vertices;
    const uint32_t *comp = stats->components;
    const uint32_t *idx = graph->vertices->edges_idx, *deg = graph->vertices->out_degree;
    const uint32_t *adj = graph->sorted_edges_array->edges_array_dest;
    /* closed under every edge, and every label is a vertex of its own class */
    uint32_t bad = 0;
#pragma omp parallel for schedule(dynamic, 1024) reduction(+ : bad)
    for (uint32_t u = 0; u < V; u++)
    {
        if (comp[u] >= V || comp[comp[u]] != comp[u]) bad++;
        for (uint32_t j = idx[u]; j < idx[u] + deg[u]; j++)
            bad += comp[adj[j]] != comp[u];
    }
    if (bad) return 0;
    /* as many classes as components (union-find), so no class joins two */
    uint32_t *p = (uint32_t *)malloc((size_t)V * 4 + 16);
    if (!p) return 0;
    for (uint32_t v = 0; v < V; v++)
        p[v] = v;
    uint32_t components = V;
    for (uint32_t u = 0; u < V; u++)
        for (uint32_t j = idx[u]; j < idx[u] + deg[u]; j++)
        {
            const uint32_t a = uf_root(p, u), b = uf_root(p, adj[j]);
            if (a != b)
            {
                p[a > b ? a : b] = a > b ? b : a;
                components--;
            }
        }
    free(p);
    uint32_t classes = 0;
    for (uint32_t v = 0; v < V; v++)
        classes += comp[v] == v;
    return classes == components ? 1u : 0u;
}
