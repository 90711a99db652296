/*
 * Host graph construction for the CSR traversal path: edge-list loaders,
 * the seeded R-MAT generator, and the CSR + inverse-CSR (CSC) build.
 *
 * The reference gets these from its OpenGraph submodule (edge-list loading,
 * radix/count sort by source with the -o flag, accel-graph.c:71-73), which is
 * absent from the snapshot; this is the project's own implementation of the
 * same contract (graphCSR.h).  The build is a parallel LSD radix sort of
 * 64-bit (key << 32 | other) words in 11-bit digits: stable, so every
 * adjacency list ends up sorted by neighbour id and the result is
 * deterministic for any thread count.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <errno.h>
#include <math.h>
#include <omp.h>

#include "graphCSR.h"
#include "gg_host.h"

#define PHI 0x9E3779B97F4A7C15ULL

static uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

static void *xmalloc(size_t n)
{
    void *p = NULL;
    if (posix_memalign(&p, 64, n ? n : 64) != 0)
        return NULL;
    return p;
}

/* ---- edge lists -------------------------------------------------------------- */

struct EdgeList *newEdgeList(uint32_t num_edges, uint32_t num_vertices, int weighted)
{
    struct EdgeList *e = (struct EdgeList *)calloc(1, sizeof(struct EdgeList));
    if (!e)
        return NULL;
    e->num_edges = num_edges;
    e->num_vertices = num_vertices;
    e->edges_array_src = (uint32_t *)xmalloc((size_t)num_edges * 4 + 64);
    e->edges_array_dest = (uint32_t *)xmalloc((size_t)num_edges * 4 + 64);
    if (weighted)
        e->edges_array_weight = (float *)xmalloc((size_t)num_edges * 4 + 64);
    if (!e->edges_array_src || !e->edges_array_dest || (weighted && !e->edges_array_weight))
    {
        freeEdgeList(e);
        return NULL;
    }
    return e;
}

void freeEdgeList(struct EdgeList *e)
{
    if (!e)
        return;
    free(e->edges_array_src);
    free(e->edges_array_dest);
    free(e->edges_array_weight);
    free(e->label_array);
    free(e->inverse_label_array);
    free(e);
}

static void finish_edge_list(struct EdgeList *e)
{
    uint32_t vmax = 0;
    float wmax = 0.0f;
    for (uint32_t i = 0; i < e->num_edges; i++)
    {
        if (e->edges_array_src[i] > vmax) vmax = e->edges_array_src[i];
        if (e->edges_array_dest[i] > vmax) vmax = e->edges_array_dest[i];
        if (e->edges_array_weight && e->edges_array_weight[i] > wmax) wmax = e->edges_array_weight[i];
    }
    e->num_vertices = e->num_edges ? vmax + 1 : 0;
    e->max_weight = wmax;
}

struct EdgeList *readEdgeListsbin(const char *fname, int weighted)
{
    FILE *f = fopen(fname, "rb");
    if (!f)
    {
        fprintf(stderr, "readEdgeListsbin: cannot open %s: %s\n", fname, strerror(errno));
        return NULL;
    }
    fseek(f, 0, SEEK_END);
    long bytes = ftell(f);
    fseek(f, 0, SEEK_SET);
    const size_t rec = weighted ? 12 : 8;
    if (bytes < 0 || (size_t)bytes % rec != 0)
    {
        fprintf(stderr, "readEdgeListsbin: %s: size %ld is not a multiple of %zu\n", fname, bytes, rec);
        fclose(f);
        return NULL;
    }
    if ((size_t)bytes / rec > 0xffffffffull)
    {
        fprintf(stderr, "readEdgeListsbin: %s: more than 2^32-1 edges\n", fname);
        fclose(f);
        return NULL;
    }
    uint32_t n = (uint32_t)((size_t)bytes / rec);
    struct EdgeList *e = newEdgeList(n, 0, weighted);
    uint32_t *buf = (uint32_t *)xmalloc((size_t)bytes + 16);
    if (!e || !buf || fread(buf, 1, (size_t)bytes, f) != (size_t)bytes)
    {
        fprintf(stderr, "readEdgeListsbin: %s: read failed\n", fname);
        free(buf);
        freeEdgeList(e);
        fclose(f);
        return NULL;
    }
    fclose(f);
    const uint32_t k = weighted ? 3 : 2;
    for (uint32_t i = 0; i < n; i++)
    {
        e->edges_array_src[i] = buf[(size_t)i * k];
        e->edges_array_dest[i] = buf[(size_t)i * k + 1];
        if (weighted)
            e->edges_array_weight[i] = (float)buf[(size_t)i * k + 2];
    }
    free(buf);
    finish_edge_list(e);
    return e;
}

struct EdgeList *readEdgeListsText(const char *fname, int weighted)
{
    FILE *f = fopen(fname, "r");
    if (!f)
    {
        fprintf(stderr, "readEdgeListsText: cannot open %s: %s\n", fname, strerror(errno));
        return NULL;
    }
    /* one edge per line: "src dst" or "src dst weight"; lines that do not
     * start with two numbers (comments, headers, blank lines) are skipped */
    size_t cap = 1024;
    uint32_t n = 0;
    uint32_t *s = (uint32_t *)malloc(cap * 4), *d = (uint32_t *)malloc(cap * 4);
    float *w = weighted ? (float *)malloc(cap * 4) : NULL;
    int ok = s && d && (!weighted || w);
    char line[512];
    while (ok && fgets(line, sizeof line, f))
    {
        unsigned long a, b;
        double c = 1.0;
        int got = sscanf(line, "%lu %lu %lf", &a, &b, &c);
        if (got < 2)
            continue;
        if (n == 0xffffffffu)
        {
            fprintf(stderr, "readEdgeListsText: %s: more than 2^32-1 edges\n", fname);
            ok = 0;
            break;
        }
        if (n == cap)
        {
            cap *= 2;
            uint32_t *s2 = (uint32_t *)realloc(s, cap * 4);
            if (s2) s = s2;
            uint32_t *d2 = (uint32_t *)realloc(d, cap * 4);
            if (d2) d = d2;
            float *w2 = w ? (float *)realloc(w, cap * 4) : NULL;
            if (w2) w = w2;
            if (!s2 || !d2 || (weighted && !w2))
            {
                fprintf(stderr, "readEdgeListsText: %s: out of memory\n", fname);
                ok = 0;
                break;
            }
        }
        s[n] = (uint32_t)a;
        d[n] = (uint32_t)b;
        if (w) w[n] = (float)(got >= 3 ? c : 1.0);
        n++;
    }
    fclose(f);
    struct EdgeList *e = ok ? newEdgeList(n, 0, weighted) : NULL;
    if (e)
    {
        memcpy(e->edges_array_src, s, (size_t)n * 4);
        memcpy(e->edges_array_dest, d, (size_t)n * 4);
        if (w) memcpy(e->edges_array_weight, w, (size_t)n * 4);
        finish_edge_list(e);
    }
    free(s);
    free(d);
    free(w);
    return e;
}

/* edge i of the R-MAT graph of 2^scale vertices drawn with `seed` */
static inline void rmat_edge(uint64_t seed, uint64_t i, uint32_t scale, double t1, double t2, double t3,
                             uint32_t *src, uint32_t *dst)
{
    uint32_t s = 0, d = 0;
    for (uint32_t l = 0; l < scale; l++)
    {
        const uint64_t r = mix64(seed + (i * scale + l + 1) * PHI);
        const double u = (double)(r >> 11) * (1.0 / 9007199254740992.0);
        const uint32_t bit = 1u << (scale - 1 - l);
        if (u < t1) { }
        else if (u < t2) d |= bit;
        else if (u < t3) s |= bit;
        else { s |= bit; d |= bit; }
    }
    *src = s;
    *dst = d;
}

struct EdgeList *generateRMATEdgeList(uint32_t scale, uint32_t edge_factor, double a, double b, double c,
                                      uint64_t seed, int weighted, uint64_t weight_seed, int symmetric)
{
    if (scale == 0 || scale > 31)
        return NULL;
    const uint64_t V = 1ull << scale;
    const uint64_t E0 = V * edge_factor;
    const uint64_t E = symmetric ? 2 * E0 : E0;
    if (E >= 0xffffffffull)
    {
        fprintf(stderr, "generateRMATEdgeList: %llu edges do not fit 32-bit offsets\n", (unsigned long long)E);
        return NULL;
    }
    struct EdgeList *e = newEdgeList((uint32_t)E, (uint32_t)V, weighted);
    if (!e)
        return NULL;
    const double t1 = a, t2 = a + b, t3 = a + b + c;
    uint32_t *src = e->edges_array_src, *dst = e->edges_array_dest;
    float *w = e->edges_array_weight;
#pragma omp parallel for schedule(static)
    for (uint64_t i = 0; i < E0; i++)
    {
        uint32_t s, d;
        rmat_edge(seed, i, scale, t1, t2, t3, &s, &d);
        src[i] = s;
        dst[i] = d;
        if (symmetric)
        {
            src[E0 + i] = d;
            dst[E0 + i] = s;
        }
        if (w)
        {
            const uint64_t r = mix64(weight_seed + (i + 1) * PHI);
            const float wv = (float)((double)(r >> 40) * (1.0 / 16777216.0));
            w[i] = wv;
            if (symmetric) w[E0 + i] = wv;
        }
    }
    e->num_vertices = (uint32_t)V;
    float wmax = 0.0f;
    if (w)
        for (uint64_t i = 0; i < E; i++)
            if (w[i] > wmax) wmax = w[i];
    e->max_weight = wmax;
    return e;
}

struct EdgeList *generateRMATBatchEdgeList(uint32_t ngraphs, const uint32_t *scales, uint32_t edge_factor, double a,
                                           double b, double c, uint64_t seed0, uint32_t *vertex_off)
{
    if (!scales || !vertex_off)
        return NULL;
    uint64_t *eoff = (uint64_t *)malloc(((size_t)ngraphs + 1) * sizeof(uint64_t));
    if (!eoff)
        return NULL;
    uint64_t V = 0, E = 0;
    eoff[0] = 0;
    for (uint32_t g = 0; g < ngraphs; g++)
    {
        if (scales[g] == 0 || scales[g] > 31)
        {
            free(eoff);
            return NULL;
        }
        vertex_off[g] = (uint32_t)V;
        V += 1ull << scales[g];
        E += (1ull << scales[g]) * edge_factor;
        eoff[g + 1] = E;
        if (V >= 0xffffffffull || E >= 0xffffffffull)
        {
            fprintf(stderr, "generateRMATBatchEdgeList: %llu vertices / %llu edges do not fit 32-bit ids\n",
                    (unsigned long long)V, (unsigned long long)E);
            free(eoff);
            return NULL;
        }
    }
    vertex_off[ngraphs] = (uint32_t)V;
    struct EdgeList *e = newEdgeList((uint32_t)E, (uint32_t)V, 0);
    if (!e)
    {
        free(eoff);
        return NULL;
    }
    const double t1 = a, t2 = a + b, t3 = a + b + c;
    uint32_t *src = e->edges_array_src, *dst = e->edges_array_dest;
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t g = 0; g < (int64_t)ngraphs; g++)
    {
        const uint32_t base = vertex_off[g], sc = scales[g];
        const uint64_t n = eoff[g + 1] - eoff[g];
        uint32_t *sp = src + eoff[g], *dp = dst + eoff[g];
        for (uint64_t i = 0; i < n; i++)
        {
            uint32_t s, d;
            rmat_edge(seed0 + (uint64_t)g, i, sc, t1, t2, t3, &s, &d);
            sp[i] = base + s;
            dp[i] = base + d;
        }
    }
    e->num_vertices = (uint32_t)V;
    free(eoff);
    return e;
}

/* ---- parallel stable LSD radix sort of 64-bit words with a float payload ----- */

#define RDX_BITS 11
#define RDX_SIZE (1u << RDX_BITS)

static void radix_sort64(uint64_t *keys, uint64_t *tmp, float *pay, float *ptmp, size_t n, int key_bits)
{
    const int passes = (key_bits + RDX_BITS - 1) / RDX_BITS;
    int T = omp_get_max_threads();
    if (T < 1) T = 1;
    if ((size_t)T > n / 4096 + 1) T = (int)(n / 4096 + 1);
    size_t *hist = (size_t *)calloc((size_t)T * RDX_SIZE, sizeof(size_t));
    for (int p = 0; p < passes; p++)
    {
        const int shift = p * RDX_BITS;
        memset(hist, 0, (size_t)T * RDX_SIZE * sizeof(size_t));
#pragma omp parallel num_threads(T)
        {
            const int t = omp_get_thread_num();
            const size_t lo = n * (size_t)t / (size_t)T, hi = n * (size_t)(t + 1) / (size_t)T;
            size_t *h = hist + (size_t)t * RDX_SIZE;
            for (size_t i = lo; i < hi; i++)
                h[(keys[i] >> shift) & (RDX_SIZE - 1)]++;
#pragma omp barrier
#pragma omp single
            {
                size_t run = 0;
                for (uint32_t d = 0; d < RDX_SIZE; d++)
                    for (int tt = 0; tt < T; tt++)
                    {
                        size_t c = hist[(size_t)tt * RDX_SIZE + d];
                        hist[(size_t)tt * RDX_SIZE + d] = run;
                        run += c;
                    }
            }
            for (size_t i = lo; i < hi; i++)
            {
                const size_t at = h[(keys[i] >> shift) & (RDX_SIZE - 1)]++;
                tmp[at] = keys[i];
                if (pay)
                    ptmp[at] = pay[i];
            }
        }
        uint64_t *k2 = keys; keys = tmp; tmp = k2;
        float *p2 = pay; pay = ptmp; ptmp = p2;
    }
    if (passes & 1)
    {
        /* result is in the scratch buffers: copy back */
#pragma omp parallel for schedule(static)
        for (size_t i = 0; i < n; i++)
        {
            tmp[i] = keys[i];
            if (pay)
                ptmp[i] = pay[i];
        }
    }
    free(hist);
}

static int bits_for(uint32_t V)
{
    int b = 1;
    while (b < 32 && (1ull << b) < V)
        b++;
    return b;
}

/* One direction: CSR keyed by `key` (lists sorted by `other`). */
static int build_direction(uint32_t V, uint32_t E, const uint32_t *key, const uint32_t *other, const float *w,
                           struct Vertex *vx, struct EdgeList *el)
{
    uint64_t *k = (uint64_t *)xmalloc((size_t)E * 8 + 64), *t = (uint64_t *)xmalloc((size_t)E * 8 + 64);
    float *pw = NULL, *pt = NULL;
    if (w)
    {
        pw = (float *)xmalloc((size_t)E * 4 + 64);
        pt = (float *)xmalloc((size_t)E * 4 + 64);
    }
    if (!k || !t || (w && (!pw || !pt)))
    {
        free(k); free(t); free(pw); free(pt);
        return -1;
    }
    /* word = key in the high b bits, other in the low b bits: the radix
     * digits cover 2b bits, low (other) digits first, so the sort is by key
     * and then by other */
    const int b = bits_for(V);
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < E; i++)
    {
        k[i] = ((uint64_t)key[i] << b) | other[i];
        if (w) pw[i] = w[i];
    }
    radix_sort64(k, t, pw, pt, E, 2 * b);
    const uint64_t lowmask = (1ull << b) - 1;
    /* edges_idx[v] = first position whose key is >= v (binary search) */
#pragma omp parallel for schedule(static)
    for (uint32_t v = 0; v < V; v++)
    {
        size_t lo = 0, hi = E;
        while (lo < hi)
        {
            size_t mid = (lo + hi) >> 1;
            if ((k[mid] >> b) < v) lo = mid + 1; else hi = mid;
        }
        vx->edges_idx[v] = (uint32_t)lo;
    }
#pragma omp parallel for schedule(static)
    for (uint32_t v = 0; v < V; v++)
        vx->out_degree[v] = (v + 1 < V ? vx->edges_idx[v + 1] : E) - vx->edges_idx[v];
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < E; i++)
    {
        el->edges_array_src[i] = (uint32_t)(k[i] >> b);
        el->edges_array_dest[i] = (uint32_t)(k[i] & lowmask);
        if (w) el->edges_array_weight[i] = pw[i];
    }
    free(k); free(t); free(pw); free(pt);
    return 0;
}

static struct Vertex *new_vertex(uint32_t V)
{
    struct Vertex *v = (struct Vertex *)calloc(1, sizeof(struct Vertex));
    if (!v) return NULL;
    v->out_degree = (uint32_t *)xmalloc((size_t)V * 4 + 64);
    v->in_degree = (uint32_t *)xmalloc((size_t)V * 4 + 64);
    v->edges_idx = (uint32_t *)xmalloc((size_t)V * 4 + 64);
    return v;
}

static void free_vertex(struct Vertex *v)
{
    if (!v) return;
    gg_host_unpin(v->out_degree);
    gg_host_unpin(v->in_degree);
    gg_host_unpin(v->edges_idx);
    free(v->out_degree);
    free(v->in_degree);
    free(v->edges_idx);
    free(v);
}

static void free_edges(struct EdgeList *e)
{
    if (!e) return;
    gg_host_unpin(e->edges_array_src);
    gg_host_unpin(e->edges_array_dest);
    gg_host_unpin(e->edges_array_weight);
    freeEdgeList(e);
}

/* the GraphCSR shell both builds fill: vertex arrays and the two sorted
 * edge lists, sized for V and E */
static struct GraphCSR *alloc_graph(uint32_t V, uint32_t E, int weighted, float max_weight)
{
    struct GraphCSR *g = (struct GraphCSR *)calloc(1, sizeof(struct GraphCSR));
    if (!g)
        return NULL;
    g->num_vertices = V;
    g->num_edges = E;
    g->max_weight = max_weight;
    g->avg_degree = V ? E / V : 0;
    g->vertices = new_vertex(V);
    g->inverse_vertices = new_vertex(V);
    g->sorted_edges_array = newEdgeList(E, V, weighted);
    g->inverse_sorted_edges_array = newEdgeList(E, V, weighted);
    if (!g->vertices || !g->inverse_vertices || !g->sorted_edges_array || !g->inverse_sorted_edges_array)
    {
        graphCSRFree(g);
        return NULL;
    }
    return g;
}

/* degrees across directions, identity labels, page-locking for upload */
static struct GraphCSR *finish_graph(struct GraphCSR *g)
{
    const uint32_t V = g->num_vertices, E = g->num_edges;
    const int weighted = g->sorted_edges_array->edges_array_weight != NULL;
    /* the inverse direction stores (dst, src): edges_array_src holds the
     * destination and edges_array_dest the in-neighbour, as the reference's
     * inverse_sorted_edges_array does */
    memcpy(g->vertices->in_degree, g->inverse_vertices->out_degree, (size_t)V * 4);
    memcpy(g->inverse_vertices->in_degree, g->vertices->out_degree, (size_t)V * 4);
    for (int d = 0; d < 2; d++)
    {
        struct EdgeList *el = d ? g->inverse_sorted_edges_array : g->sorted_edges_array;
        el->num_vertices = V;
        el->max_weight = g->max_weight;
        el->label_array = (uint32_t *)xmalloc((size_t)V * 4 + 64);
        el->inverse_label_array = (uint32_t *)xmalloc((size_t)V * 4 + 64);
        if (!el->label_array || !el->inverse_label_array)
        {
            graphCSRFree(g);
            return NULL;
        }
        for (uint32_t v = 0; v < V; v++)
            el->label_array[v] = el->inverse_label_array[v] = v;
    }
    /* page-lock the arrays the GPU path uploads (no-op without a device) */
    gg_host_pin(g->vertices->out_degree, (size_t)V * 4);
    gg_host_pin(g->vertices->edges_idx, (size_t)V * 4);
    gg_host_pin(g->inverse_vertices->edges_idx, (size_t)V * 4);
    gg_host_pin(g->sorted_edges_array->edges_array_dest, (size_t)E * 4);
    gg_host_pin(g->inverse_sorted_edges_array->edges_array_dest, (size_t)E * 4);
    if (weighted)
    {
        gg_host_pin(g->sorted_edges_array->edges_array_weight, (size_t)E * 4);
        gg_host_pin(g->inverse_sorted_edges_array->edges_array_weight, (size_t)E * 4);
    }
    return g;
}

struct GraphCSR *graphCSRFromEdgeList(const struct EdgeList *in)
{
    if (!in)
        return NULL;
    const uint32_t V = in->num_vertices, E = in->num_edges;
    const int weighted = in->edges_array_weight != NULL;
    struct GraphCSR *g = alloc_graph(V, E, weighted, in->max_weight);
    if (!g)
        return NULL;
    if (build_direction(V, E, in->edges_array_src, in->edges_array_dest, in->edges_array_weight, g->vertices,
                        g->sorted_edges_array) != 0 ||
        build_direction(V, E, in->edges_array_dest, in->edges_array_src, in->edges_array_weight,
                        g->inverse_vertices, g->inverse_sorted_edges_array) != 0)
    {
        graphCSRFree(g);
        return NULL;
    }
    return finish_graph(g);
}

/* rows and degrees of one direction from its offsets */
static void rows_from_offsets(uint32_t V, uint32_t E, const uint32_t *idx, uint32_t *row, uint32_t *deg)
{
#pragma omp parallel for schedule(dynamic, 4096)
    for (uint32_t v = 0; v < V; v++)
    {
        const uint32_t a = idx[v], b = v + 1 < V ? idx[v + 1] : E;
        deg[v] = b - a;
        for (uint32_t i = a; i < b; i++)
            row[i] = v;
    }
}

/* the device build, copied back; with `labels` (orig -> new) the edge list
 * is relabelled first and the label arrays record the mapping */
static struct GraphCSR *device_build(const struct EdgeList *in, const uint32_t *labels, const char *who)
{
    const uint32_t V = in->num_vertices, E = in->num_edges;
    const int weighted = in->edges_array_weight != NULL;
    gg_graph *d = NULL;
    const uint32_t what = GG_MAP_OUT | GG_MAP_IN | (weighted ? (GG_MAP_OUT_W | GG_MAP_IN_W) : 0u);
    gg_status bst = labels ? gg_graph_build_relabelled(in, labels, what, NULL, &d) : gg_graph_build(in, what, NULL, &d);
    if (bst != GG_OK)
    {
        gpu_report(who, bst);
        return NULL;
    }
    struct GraphCSR *g = alloc_graph(V, E, weighted, in->max_weight);
    if (!g)
    {
        gg_graph_unmap(d);
        return NULL;
    }
    struct EdgeList *fw = g->sorted_edges_array, *bw = g->inverse_sorted_edges_array;
    gg_status st = gg_graph_download(d, g->vertices->edges_idx, fw->edges_array_dest, fw->edges_array_weight,
                                     g->inverse_vertices->edges_idx, bw->edges_array_dest, bw->edges_array_weight, NULL);
    gg_graph_unmap(d);
    if (st != GG_OK)
    {
        gpu_report(who, st);
        graphCSRFree(g);
        return NULL;
    }
    rows_from_offsets(V, E, g->vertices->edges_idx, fw->edges_array_src, g->vertices->out_degree);
    rows_from_offsets(V, E, g->inverse_vertices->edges_idx, bw->edges_array_src, g->inverse_vertices->out_degree);
    g = finish_graph(g);
    if (g && labels)
        for (int k = 0; k < 2; k++)
        {
            struct EdgeList *el = k ? bw : fw;
            for (uint32_t v = 0; v < V; v++)
            {
                el->label_array[v] = labels[v];
                el->inverse_label_array[labels[v]] = v;
            }
        }
    return g;
}

struct GraphCSR *graphCSRFromEdgeListDevice(const struct EdgeList *in)
{
    if (!in)
        return NULL;
    return device_build(in, NULL, "graphCSRFromEdgeListDevice");
}

struct GraphCSR *graphCSRFromEdgeListRelabelDevice(const struct EdgeList *in, uint32_t lmode, uint64_t seed)
{
    if (!in)
        return NULL;
    uint32_t *labels = (uint32_t *)malloc((size_t)in->num_vertices * 4 + 16);
    if (!labels)
        return NULL;
    gg_status st = gg_relabel_order(in, lmode, seed, labels, NULL);
    struct GraphCSR *g = NULL;
    if (st != GG_OK)
        gpu_report("graphCSRFromEdgeListRelabelDevice", st);
    else
        g = device_build(in, labels, "graphCSRFromEdgeListRelabelDevice");
    free(labels);
    return g;
}

void graphCSRFree(struct GraphCSR *g)
{
    if (!g)
        return;
    free_vertex(g->vertices);
    free_vertex(g->inverse_vertices);
    free_edges(g->sorted_edges_array);
    free_edges(g->inverse_sorted_edges_array);
    free(g);
}

/* ---- serialisation: the reference's -z / -c / -x formats ------------------------
 * (02_capi_graph/src/main/accel-graph.c:51 -z, :115-128 -c, :339-341 -x).
 * Text and binary edge lists are the 04_test_graphs formats; the graphCSR
 * binary layout is OpenGraph's and that code is absent, so this one is the
 * project's own: a header, then every array of the GraphCSR in a fixed
 * order, so a read gives back a graph whose arrays equal the written ones. */

static int write_all(FILE *f, const void *p, size_t n) { return n == 0 || fwrite(p, 1, n, f) == n; }
static int read_all(FILE *f, void *p, size_t n) { return n == 0 || fread(p, 1, n, f) == n; }

int writeEdgeListsText(const struct EdgeList *e, const char *fname)
{
    FILE *f = e ? fopen(fname, "w") : NULL;
    if (!f)
    {
        fprintf(stderr, "writeEdgeListsText: cannot open %s: %s\n", fname, e ? strerror(errno) : "no edge list");
        return -1;
    }
    int ok = 1;
    for (uint32_t i = 0; ok && i < e->num_edges; i++)
    {
        if (e->edges_array_weight)
            ok = fprintf(f, "%u %u %.9g\n", e->edges_array_src[i], e->edges_array_dest[i],
                         (double)e->edges_array_weight[i]) > 0;
        else
            ok = fprintf(f, "%u %u\n", e->edges_array_src[i], e->edges_array_dest[i]) > 0;
    }
    ok = (fclose(f) == 0) && ok;
    if (!ok) fprintf(stderr, "writeEdgeListsText: %s: write failed\n", fname);
    return ok ? 0 : -1;
}

int writeEdgeListsbin(const struct EdgeList *e, const char *fname)
{
    FILE *f = e ? fopen(fname, "wb") : NULL;
    if (!f)
    {
        fprintf(stderr, "writeEdgeListsbin: cannot open %s: %s\n", fname, e ? strerror(errno) : "no edge list");
        return -1;
    }
    const int weighted = e->edges_array_weight != NULL;
    const uint32_t k = weighted ? 3 : 2, chunk = 1u << 16;
    uint32_t *buf = (uint32_t *)xmalloc((size_t)chunk * k * 4);
    int ok = buf != NULL;
    for (uint32_t i0 = 0; ok && i0 < e->num_edges; i0 += chunk)
    {
        const uint32_t n = e->num_edges - i0 < chunk ? e->num_edges - i0 : chunk;
        for (uint32_t j = 0; j < n; j++)
        {
            buf[(size_t)j * k] = e->edges_array_src[i0 + j];
            buf[(size_t)j * k + 1] = e->edges_array_dest[i0 + j];
            /* the weight word is an integer, as readEdgeListsbin reads it */
            if (weighted) buf[(size_t)j * k + 2] = (uint32_t)lrintf(e->edges_array_weight[i0 + j]);
        }
        ok = write_all(f, buf, (size_t)n * k * 4);
    }
    free(buf);
    ok = (fclose(f) == 0) && ok;
    if (!ok) fprintf(stderr, "writeEdgeListsbin: %s: write failed\n", fname);
    return ok ? 0 : -1;
}

#define GG_CSR_MAGIC "AGXCSR1"

struct csr_file_header
{
    char magic[8];
    uint32_t num_vertices, num_edges, weighted, avg_degree;
    float max_weight;
    uint32_t reserved[3];
};

/* the arrays of a GraphCSR in file order: (pointer, element count) */
static int csr_arrays(const struct GraphCSR *g, void **ptr, size_t *n)
{
    const size_t V = g->num_vertices, E = g->num_edges;
    int k = 0;
    const struct Vertex *vx[2] = {g->vertices, g->inverse_vertices};
    for (int d = 0; d < 2; d++)
    {
        ptr[k] = vx[d]->out_degree; n[k++] = V;
        ptr[k] = vx[d]->in_degree; n[k++] = V;
        ptr[k] = vx[d]->edges_idx; n[k++] = V;
    }
    const struct EdgeList *el[2] = {g->sorted_edges_array, g->inverse_sorted_edges_array};
    for (int d = 0; d < 2; d++)
    {
        ptr[k] = el[d]->edges_array_src; n[k++] = E;
        ptr[k] = el[d]->edges_array_dest; n[k++] = E;
        ptr[k] = el[d]->edges_array_weight; n[k++] = el[d]->edges_array_weight ? E : 0;
        ptr[k] = el[d]->label_array; n[k++] = V;
        ptr[k] = el[d]->inverse_label_array; n[k++] = V;
    }
    return k;
}

int writeGraphCSRbin(const struct GraphCSR *g, const char *fname)
{
    FILE *f = g ? fopen(fname, "wb") : NULL;
    if (!f)
    {
        fprintf(stderr, "writeGraphCSRbin: cannot open %s: %s\n", fname, g ? strerror(errno) : "no graph");
        return -1;
    }
    struct csr_file_header h;
    memset(&h, 0, sizeof h);
    memcpy(h.magic, GG_CSR_MAGIC, 8);
    h.num_vertices = g->num_vertices;
    h.num_edges = g->num_edges;
    h.weighted = g->sorted_edges_array->edges_array_weight != NULL;
    h.avg_degree = g->avg_degree;
    h.max_weight = g->max_weight;
    void *ptr[16];
    size_t n[16];
    const int na = csr_arrays(g, ptr, n);
    int ok = write_all(f, &h, sizeof h);
    for (int i = 0; ok && i < na; i++)
        ok = write_all(f, ptr[i], n[i] * 4);
    ok = (fclose(f) == 0) && ok;
    if (!ok) fprintf(stderr, "writeGraphCSRbin: %s: write failed\n", fname);
    return ok ? 0 : -1;
}

struct GraphCSR *readGraphCSRbin(const char *fname)
{
    FILE *f = fopen(fname, "rb");
    if (!f)
    {
        fprintf(stderr, "readGraphCSRbin: cannot open %s: %s\n", fname, strerror(errno));
        return NULL;
    }
    struct csr_file_header h;
    if (!read_all(f, &h, sizeof h) || memcmp(h.magic, GG_CSR_MAGIC, 8) != 0)
    {
        fprintf(stderr, "readGraphCSRbin: %s: not a graphCSR binary file\n", fname);
        fclose(f);
        return NULL;
    }
    fseek(f, 0, SEEK_END);
    const long bytes = ftell(f);
    const uint64_t want = sizeof h + 4ull * (10ull * h.num_vertices + 4ull * h.num_edges +
                                             (h.weighted ? 2ull * h.num_edges : 0ull));
    if (bytes < 0 || (uint64_t)bytes != want)
    {
        fprintf(stderr, "readGraphCSRbin: %s: size %ld, expected %llu\n", fname, bytes, (unsigned long long)want);
        fclose(f);
        return NULL;
    }
    fseek(f, (long)sizeof h, SEEK_SET);
    struct GraphCSR *g = alloc_graph(h.num_vertices, h.num_edges, h.weighted != 0, h.max_weight);
    int ok = g != NULL;
    for (int d = 0; ok && d < 2; d++)
    {
        struct EdgeList *el = d ? g->inverse_sorted_edges_array : g->sorted_edges_array;
        el->label_array = (uint32_t *)xmalloc((size_t)h.num_vertices * 4 + 64);
        el->inverse_label_array = (uint32_t *)xmalloc((size_t)h.num_vertices * 4 + 64);
        el->max_weight = h.max_weight;
        ok = el->label_array && el->inverse_label_array;
    }
    void *ptr[16];
    size_t n[16];
    const int na = ok ? csr_arrays(g, ptr, n) : 0;
    for (int i = 0; ok && i < na; i++)
        ok = read_all(f, ptr[i], n[i] * 4);
    fclose(f);
    if (!ok)
    {
        fprintf(stderr, "readGraphCSRbin: %s: read failed\n", fname);
        graphCSRFree(g);
        return NULL;
    }
    g->avg_degree = h.avg_degree;
    /* page-lock the arrays the GPU path uploads, as the builds do */
    const size_t V = h.num_vertices, E = h.num_edges;
    gg_host_pin(g->vertices->out_degree, V * 4);
    gg_host_pin(g->vertices->edges_idx, V * 4);
    gg_host_pin(g->inverse_vertices->edges_idx, V * 4);
    gg_host_pin(g->sorted_edges_array->edges_array_dest, E * 4);
    gg_host_pin(g->inverse_sorted_edges_array->edges_array_dest, E * 4);
    if (h.weighted)
    {
        gg_host_pin(g->sorted_edges_array->edges_array_weight, E * 4);
        gg_host_pin(g->inverse_sorted_edges_array->edges_array_weight, E * 4);
    }
    return g;
}

struct EdgeList *edgeListFromGraphCSR(const struct GraphCSR *g)
{
    if (!g)
        return NULL;
    const struct EdgeList *s = g->sorted_edges_array;
    struct EdgeList *e = newEdgeList(g->num_edges, g->num_vertices, s->edges_array_weight != NULL);
    if (!e)
        return NULL;
    /* edges in CSR order, as original ids (through the inverse labels) */
    for (uint32_t i = 0; i < g->num_edges; i++)
    {
        e->edges_array_src[i] = s->inverse_label_array[s->edges_array_src[i]];
        e->edges_array_dest[i] = s->inverse_label_array[s->edges_array_dest[i]];
        if (e->edges_array_weight) e->edges_array_weight[i] = s->edges_array_weight[i];
    }
    e->num_vertices = g->num_vertices;
    e->max_weight = g->max_weight;
    return e;
}

struct GraphCSR *graphCSRFromFile(const char *fname, uint32_t format, int weighted)
{
    if (format == 2)
        return readGraphCSRbin(fname);
    struct EdgeList *e = format == 0 ? readEdgeListsText(fname, weighted) : readEdgeListsbin(fname, weighted);
    if (!e)
        return NULL;
    struct GraphCSR *g = graphCSRFromEdgeList(e);
    freeEdgeList(e);
    return g;
}

void writeSerializedGraphDataStructure(struct Arguments *arguments)
{
    if (!arguments || !arguments->fnameb)
    {
        fprintf(stderr, "writeSerializedGraphDataStructure: no input file (-f)\n");
        return;
    }
    const char *in = arguments->fnameb;
    const uint32_t from = arguments->fnameb_format, to = arguments->convert_format;
    const int weighted = arguments->weighted != 0;
    const char *ext = to == 0 ? ".txt" : to == 1 ? (weighted ? ".wbin" : ".bin") : ".csr";
    size_t len = strlen(in) + strlen(ext) + 1;
    char *out = (char *)malloc(len);
    if (!out)
        return;
    snprintf(out, len, "%s%s", in, ext);
    int rc = -1;
    if (to == 2)
    {
        struct GraphCSR *g = graphCSRFromFile(in, from, weighted);
        if (g) rc = writeGraphCSRbin(g, out);
        graphCSRFree(g);
    }
    else
    {
        struct EdgeList *e = NULL;
        if (from == 2)
        {
            struct GraphCSR *g = readGraphCSRbin(in);
            e = edgeListFromGraphCSR(g);
            graphCSRFree(g);
        }
        else
            e = from == 0 ? readEdgeListsText(in, weighted) : readEdgeListsbin(in, weighted);
        if (e) rc = to == 0 ? writeEdgeListsText(e, out) : writeEdgeListsbin(e, out);
        freeEdgeList(e);
    }
    if (rc == 0)
        printf("| %-51s | \n| %-51s | \n", "serialised", out);
    else
        fprintf(stderr, "writeSerializedGraphDataStructure: %s -> %s failed\n", in, out);
    free(out);
}
