/*
 * CPU oracle for the CSR traversal hot path -- TEST INFRASTRUCTURE ONLY.
 * See oracle.h for what it is, what pins it and who may call it.
 *
 * Build: oracle/Makefile (gcc -O2 -ffp-contract=off -fopenmp).  FP
 * contraction is off so that `a + b*c` rounds twice, as the reference's C
 * does on a target without fused multiply-add, on every host architecture.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PHI 0x9E3779B97F4A7C15ULL

/* ------------------------------------------------------------------------ */
/* graph construction                                                        */
/* ------------------------------------------------------------------------ */

uint64_t orc_splitmix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

void orc_rmat_edges(uint32_t scale, double a, double b, double c, uint64_t seed,
                    uint64_t first, uint64_t count, uint32_t *src, uint32_t *dst)
{
    const double t1 = a, t2 = a + b, t3 = a + b + c;
    /* every edge is a function of its index alone: any schedule gives the
     * same list */
#pragma omp parallel for schedule(static)
    for (uint64_t k = 0; k < count; k++)
    {
        uint64_t i = first + k;
        uint32_t s = 0, d = 0;
        for (uint32_t l = 0; l < scale; l++)
        {
            uint64_t r = orc_splitmix64(seed + (i * scale + l + 1) * PHI);
            double u = (double)(r >> 11) * (1.0 / 9007199254740992.0);
            uint32_t bit = 1u << (scale - 1 - l);
            if (u < t1) { }
            else if (u < t2) d |= bit;
            else if (u < t3) s |= bit;
            else { s |= bit; d |= bit; }
        }
        src[k] = s;
        dst[k] = d;
    }
}

void orc_rmat_weights(uint64_t seed, uint64_t first, uint64_t count, float *w)
{
#pragma omp parallel for schedule(static)
    for (uint64_t k = 0; k < count; k++)
    {
        uint64_t r = orc_splitmix64(seed + (first + k + 1) * PHI);
        w[k] = (float)((double)(r >> 40) * (1.0 / 16777216.0));
    }
}

/* Stable LSD radix sort of (key, val) pairs on the low `bits` bits of key,
 * 8 bits per pass, OpenMP: each thread histograms and scatters its own
 * contiguous chunk, chunks in thread order, so equal digits keep their input
 * order (stable) whatever the thread count.  The result ends in key/val. */
static void radix_sort_pairs(uint64_t *key, uint32_t *val, size_t n, int bits)
{
    uint64_t *k2 = (uint64_t *)malloc(n * sizeof(uint64_t) + 8);
    uint32_t *v2 = (uint32_t *)malloc(n * sizeof(uint32_t) + 4);
    int nt = 1;
#ifdef _OPENMP
    nt = omp_get_max_threads();
#endif
    size_t *cnt = (size_t *)malloc((size_t)nt * 256 * sizeof(size_t));
    uint64_t *ka = key, *kb = k2;
    uint32_t *va = val, *vb = v2;
    for (int shift = 0; shift < bits; shift += 8)
    {
#pragma omp parallel num_threads(nt)
        {
            int t = 0;
#ifdef _OPENMP
            t = omp_get_thread_num();
#endif
            const size_t lo = n * (size_t)t / (size_t)nt, hi = n * (size_t)(t + 1) / (size_t)nt;
            size_t *c = cnt + (size_t)t * 256;
            memset(c, 0, 256 * sizeof(size_t));
            for (size_t i = lo; i < hi; i++)
                c[(ka[i] >> shift) & 255]++;
#pragma omp barrier
#pragma omp single
            {
                size_t run = 0;
                for (int d = 0; d < 256; d++)
                    for (int u = 0; u < nt; u++)
                    {
                        size_t x = cnt[(size_t)u * 256 + d];
                        cnt[(size_t)u * 256 + d] = run;
                        run += x;
                    }
            }
            for (size_t i = lo; i < hi; i++)
            {
                size_t at = c[(ka[i] >> shift) & 255]++;
                kb[at] = ka[i];
                vb[at] = va[i];
            }
        }
        uint64_t *kt = ka; ka = kb; kb = kt;
        uint32_t *vt = va; va = vb; vb = vt;
    }
    if (ka != key)
    {
        memcpy(key, ka, n * sizeof(uint64_t));
        memcpy(val, va, n * sizeof(uint32_t));
    }
    free(cnt);
    free(k2);
    free(v2);
}

/* CSR (by_dst = 0) or inverse CSR (by_dst = 1) of an edge list: rows by the
 * primary endpoint, each row's neighbours ascending, duplicates (and their
 * weights) in input order -- the order of a stable sort by the neighbour
 * followed by a stable sort by the row, done here as one stable radix sort
 * of (row << b | neighbour). */
void orc_build_csr(uint32_t V, uint32_t E, const uint32_t *src, const uint32_t *dst, const float *w,
                   int by_dst, uint32_t *off, uint32_t *adj, float *adj_w)
{
    const uint32_t *primary = by_dst ? dst : src;
    const uint32_t *secondary = by_dst ? src : dst;
    int b = 1;
    while (b < 32 && ((uint64_t)1 << b) < (uint64_t)V)
        b++;
    uint64_t *key = (uint64_t *)malloc((size_t)E * sizeof(uint64_t) + 8);
    uint32_t *idx = (uint32_t *)malloc((size_t)E * sizeof(uint32_t) + 4);
#pragma omp parallel for schedule(static)
    for (uint32_t i = 0; i < E; i++)
    {
        key[i] = ((uint64_t)primary[i] << b) | secondary[i];
        idx[i] = i;
    }
    radix_sort_pairs(key, idx, E, 2 * b);
    const uint64_t mask = ((uint64_t)1 << b) - 1;
    /* off[v] = first position whose row is >= v */
#pragma omp parallel for schedule(static)
    for (uint32_t i = 0; i < E; i++)
    {
        const uint32_t r = (uint32_t)(key[i] >> b);
        const uint32_t prev = i ? (uint32_t)(key[i - 1] >> b) + 1 : 0;
        for (uint32_t v = prev; v <= r; v++)
            off[v] = i;
        adj[i] = (uint32_t)(key[i] & mask);
        if (adj_w)
            adj_w[i] = w ? w[idx[i]] : 0.0001f;
    }
    const uint32_t last = E ? (uint32_t)(key[E - 1] >> b) + 1 : 0;
    for (uint32_t v = last; v <= V; v++)
        off[v] = E;
    free(key);
    free(idx);
}

/* ------------------------------------------------------------------------ */
/* fixed point and quantisation (project formats; the reference's are in    */
/* the missing OpenGraph fixedPoint.h / quantization.h)                      */
/* ------------------------------------------------------------------------ */

uint64_t orc_fx64_from_double(double x)
{
    double t = x * 4294967296.0;
    if (!(t > 0.0))
        return 0;
    if (t >= 18446744073709551615.0)
        return UINT64_MAX;
    return (uint64_t)t;
}

double orc_fx64_to_double(uint64_t f) { return (double)f * (1.0 / 4294967296.0); }

uint64_t orc_fx64_mul(uint64_t a, uint64_t b)
{
    unsigned __int128 p = (unsigned __int128)a * (unsigned __int128)b;
    return (uint64_t)(p >> 32);
}

static uint32_t fx_from_float(float x, double scale, uint32_t maxv)
{
    double t = (double)x * scale;
    if (!(t > 0.0))
        return 0;
    if (t >= (double)maxv)
        return maxv;
    return (uint32_t)t;
}

uint32_t orc_fx32_from_float(float x) { return fx_from_float(x, 65536.0, 0xFFFFFFFFu); }
float orc_fx32_to_float(uint64_t f) { return (float)((double)f * (1.0 / 65536.0)); }
uint32_t orc_fx16_from_float(float x) { return fx_from_float(x, 4096.0, 0xFFFFu); }
float orc_fx16_to_float(uint64_t f) { return (float)((double)f * (1.0 / 4096.0)); }
uint32_t orc_fx8_from_float(float x) { return fx_from_float(x, 64.0, 0xFFu); }
float orc_fx8_to_float(uint64_t f) { return (float)((double)f * (1.0 / 64.0)); }

float orc_quant_scale(float min, float max, int bits)
{
    (void)min;
    double levels = (double)((1ull << bits) - 1);
    if (!(max > 0.0f))
        return 0.0f;
    return (float)((double)max / levels);
}

uint32_t orc_quantize(float x, float scale, uint32_t zero, int bits)
{
    double maxq = (double)((1ull << bits) - 1);
    if (scale == 0.0f)
        return zero;
    double t = floor((double)x / (double)scale + 0.5) + (double)zero;
    if (t < 0.0)
        return 0;
    if (t > maxq)
        return (uint32_t)maxq;
    return (uint32_t)t;
}

uint32_t orc_quant_zero(float max, float scale, int bits)
{
    double maxq = (double)((1ull << bits) - 1);
    if (scale == 0.0f)
        return 0;
    double t = floor(maxq - (double)max / (double)scale + 0.5);
    if (t < 0.0)
        return 0;
    if (t > maxq)
        return (uint32_t)maxq;
    return (uint32_t)t;
}

/* ------------------------------------------------------------------------ */
/* PageRank                                                                  */
/* ------------------------------------------------------------------------ */

static inline uint32_t out_degree(const orc_csr *g, uint32_t v) { return g->out_off[v + 1] - g->out_off[v]; }

/* rank / out_degree as the reference computes it (pageRank.c:1028-1031). */
static inline float contrib_of(float rank, uint32_t deg) { return deg ? rank / (float)deg : 0.0f; }

/* The shared update pass of every topology-driven variant
 * (pageRank.c:1055-1069): rank = base + damp*next, |delta| error, active. */
typedef struct upd_acc { double error_total; uint32_t active; } upd_acc;

static inline void update_vertex(float *ranks, uint32_t v, float next_rank, double epsilon, uint32_t V,
                                 upd_acc *acc)
{
    float prev = ranks[v];
    ranks[v] = next_rank;
    double error = fabs(next_rank - prev);
    acc->error_total += error / V;
    if (error >= epsilon)
        acc->active++;
}

enum { Q_BITS_PUSH = 8 };

int orc_pagerank(const orc_csr *g, int mode, uint32_t iterations, double epsilon,
                 int init_one_over_n, float *ranks, orc_pr_out *out, int nthreads)
{
    const uint32_t V = g->V;
    const float damp = 0.85f;
    const float base_pr = 1.0f - damp;
    const float base = init_one_over_n ? base_pr / (float)V : base_pr;
    if (mode < 0 || mode > 13)
        return -1;
#ifdef _OPENMP
    if (nthreads < 1)
        nthreads = 1;
#else
    (void)nthreads;
#endif

    /* newPageRankStatsGraphCSR (pageRank.c:50-78) */
    for (uint32_t v = 0; v < V; v++)
        ranks[v] = init_one_over_n ? 1.0f / (float)V : base_pr;

    float *contrib = (float *)calloc((size_t)V + 1, sizeof(float));
    float *next_f = (float *)calloc((size_t)V + 1, sizeof(float));
    uint64_t *next_u = (uint64_t *)calloc((size_t)V + 1, sizeof(uint64_t));
    uint64_t *cfx = (uint64_t *)calloc((size_t)V + 1, sizeof(uint64_t));
    uint8_t *wl_curr = (uint8_t *)calloc((size_t)V + 1, 1);
    uint8_t *wl_next = (uint8_t *)calloc((size_t)V + 1, 1);
    float *resid = (float *)calloc((size_t)V + 1, sizeof(float));

    orc_pr_out o = {0};
    upd_acc acc = {0.0, 0};
    uint32_t it = 0;
    int converged = 0;

    if (mode == 7 || mode == 8)
    {
        /* aResiduals init (pageRank.c:3013-3030) */
        for (uint32_t v = 0; v < V; v++)
        {
            float r = 0.0f;
            for (uint32_t j = g->in_off[v]; j < g->in_off[v + 1]; j++)
            {
                uint32_t u = g->in_adj[j];
                uint32_t du = out_degree(g, u);
                if (du)
                    r += 1.0f / (float)du;
            }
            resid[v] = (1.0f - damp) * damp * r;
            wl_curr[v] = 1;
        }
    }
    if (mode == 6)
        for (uint32_t v = 0; v < V; v++)
            wl_curr[v] = 1;

    for (it = 0; it < iterations; it++)
    {
        acc.error_total = 0.0;
        acc.active = 0;

        if (mode == 6)
        {
            /* data-driven pull (pageRank.c:2810-2968, loop :2880-2932) */
            for (uint32_t v = 0; v < V; v++)
                contrib[v] = contrib_of(ranks[v], out_degree(g, v));
            double err_sum = 0.0;
            uint32_t active = 0;
#pragma omp parallel for schedule(dynamic, 1024) reduction(+ : err_sum, active) num_threads(nthreads)
            for (uint32_t v = 0; v < V; v++)
            {
                if (!wl_curr[v])
                    continue;
                float in_pr = 0.0f;
                for (uint32_t j = g->in_off[v]; j < g->in_off[v + 1]; j++)
                    in_pr += contrib[g->in_adj[j]];
                float old_pr = ranks[v];
                float new_pr = base + (damp * in_pr);
                double error = fabs(new_pr - old_pr);
                err_sum += error / V;
                if (error >= epsilon)
                {
                    ranks[v] = new_pr;
                    for (uint32_t j = g->out_off[v]; j < g->out_off[v + 1]; j++)
                        wl_next[g->out_adj[j]] = 1;
                    active++;
                }
            }
            acc.error_total = err_sum;
            acc.active = active;
            uint8_t *t = wl_curr; wl_curr = wl_next; wl_next = t;
            memset(wl_next, 0, V);
        }
        else if (mode == 7 || mode == 8)
        {
            /* data-driven push / pull-push (pageRank.c:2971-3125, :3128-3300),
             * sequential order: one serialisation of the reference's racy loop */
            for (uint32_t v = 0; v < V; v++)
            {
                if (!wl_curr[v])
                    continue;
                float old_pr = ranks[v];
                float new_pr;
                if (mode == 7)
                {
                    new_pr = resid[v] + ranks[v];
                }
                else
                {
                    float in_pr = 0.0f;
                    for (uint32_t j = g->in_off[v]; j < g->in_off[v + 1]; j++)
                    {
                        uint32_t u = g->in_adj[j];
                        in_pr += ranks[u] / (float)out_degree(g, u);
                    }
                    new_pr = base + (damp * in_pr);
                }
                acc.error_total += fabs(new_pr / V - old_pr / V);
                ranks[v] = new_pr;
                uint32_t deg = out_degree(g, v);
                float delta = damp * (resid[v] / deg);
                for (uint32_t j = g->out_off[v]; j < g->out_off[v + 1]; j++)
                {
                    uint32_t u = g->out_adj[j];
                    float prev = resid[u];
                    resid[u] += delta;
                    if ((fabs(prev + delta) >= epsilon) && (prev <= epsilon))
                    {
                        acc.active++;
                        if (mode == 8)
                            resid[u] += delta;
                        wl_next[u] = 1;
                    }
                }
                resid[v] = 0.0f;
            }
            uint8_t *t = wl_curr; wl_curr = wl_next; wl_next = t;
            memset(wl_next, 0, V);
        }
        else
        {
            /* topology-driven variants: contrib pass (pageRank.c:1026-1033),
             * gather/scatter, update pass (:1055-1069) */
            float qscale = 0.0f;
            uint32_t qzero = 0;
            int qbits = 0;
            if (mode == 4 || mode == 12 || mode == 13 || mode == 5)
            {
                qbits = mode == 4 ? 32 : mode == 12 ? 16 : mode == 13 ? 8 : Q_BITS_PUSH;
                float mn = 0.0f, mx = 0.0f;
                for (uint32_t v = 0; v < V; v++)
                {
                    contrib[v] = contrib_of(ranks[v], out_degree(g, v));
                    if (v == 0 || contrib[v] < mn) mn = contrib[v];
                    if (v == 0 || contrib[v] > mx) mx = contrib[v];
                }
                qscale = orc_quant_scale(mn, mx, qbits);
                qzero = mode == 5 ? orc_quant_zero(mx, qscale, qbits) : 0;
                for (uint32_t v = 0; v < V; v++)
                    cfx[v] = orc_quantize(contrib[v], qscale, qzero, qbits);
            }
            else
            {
#pragma omp parallel for schedule(static) num_threads(nthreads)
                for (uint32_t v = 0; v < V; v++)
                {
                    uint32_t d = out_degree(g, v);
                    float c = contrib_of(ranks[v], d);
                    contrib[v] = c;
                    switch (mode)
                    {
                    case 2: case 3: cfx[v] = d ? orc_fx64_from_double(c) : 0; break;
                    case 9: cfx[v] = d ? orc_fx32_from_float(c) : 0; break;
                    case 10: cfx[v] = d ? orc_fx16_from_float(c) : 0; break;
                    case 11: cfx[v] = d ? orc_fx8_from_float(c) : 0; break;
                    default: break;
                    }
                }
            }

            int integer_sum = (mode == 2 || mode == 3 || mode == 4 || mode == 9 || mode == 10 ||
                               mode == 11 || mode == 12 || mode == 13);
            if (mode == 1 || mode == 3 || mode == 5)
            {
                /* push: scatter over out-edges (pageRank.c:2051-2065, :2741-2756) */
                for (uint32_t v = 0; v < V; v++)
                {
                    for (uint32_t j = g->out_off[v]; j < g->out_off[v + 1]; j++)
                    {
                        uint32_t u = g->out_adj[j];
                        if (mode == 1)
                            next_f[u] += contrib[v];
                        else if (mode == 3)
                            next_u[u] += cfx[v];
                        else
                            next_f[u] += qscale * (float)((int64_t)cfx[v] - (int64_t)qzero);
                    }
                }
            }
            else
            {
                /* pull: in-edge gather in CSC order, the CU's sum
                 * (cu_PageRank/CSR/PULL/.../cu_sum_kernel_control.sv:166-185) */
#pragma omp parallel for schedule(dynamic, 1024) num_threads(nthreads)
                for (uint32_t v = 0; v < V; v++)
                {
                    if (integer_sum)
                    {
                        uint64_t s = 0;
                        for (uint32_t j = g->in_off[v]; j < g->in_off[v + 1]; j++)
                            s += cfx[g->in_adj[j]];
                        next_u[v] = s;
                    }
                    else
                    {
                        float s = 0.0f;
                        for (uint32_t j = g->in_off[v]; j < g->in_off[v + 1]; j++)
                            s += contrib[g->in_adj[j]];
                        next_f[v] = s;
                    }
                }
            }

            double err_sum = 0.0;
            uint32_t active = 0;
#pragma omp parallel for reduction(+ : err_sum, active) num_threads(nthreads)
            for (uint32_t v = 0; v < V; v++)
            {
                float nr;
                switch (mode)
                {
                case 2: case 3:
                    nr = (float)((double)base + (double)damp * orc_fx64_to_double(next_u[v]));
                    break;
                case 9: nr = base + (damp * orc_fx32_to_float(next_u[v])); break;
                case 10: nr = base + (damp * orc_fx16_to_float(next_u[v])); break;
                case 11: nr = base + (damp * orc_fx8_to_float(next_u[v])); break;
                case 4: case 12: case 13:
                    nr = base + damp * (qscale * (float)next_u[v]);
                    break;
                default:
                    nr = base + (damp * next_f[v]);
                    break;
                }
                next_f[v] = 0.0f;
                next_u[v] = 0;
                upd_acc a1 = {0.0, 0};
                update_vertex(ranks, v, nr, epsilon, V, &a1);
                err_sum += a1.error_total;
                active += a1.active;
            }
            acc.error_total = err_sum;
            acc.active = active;
        }

        if (acc.active == 0)
        {
            converged = 1;
            break;
        }
    }

    /* final normalisation (pageRank.c:1080-1085) */
    double sum = 0.0;
    for (uint32_t v = 0; v < V; v++)
    {
        if (!init_one_over_n)
            ranks[v] = ranks[v] / (float)V;
        sum += ranks[v];
    }
    o.iterations = it;
    o.active = acc.active;
    o.error_total = acc.error_total;
    o.rank_sum = sum;
    o.executed = converged ? it + 1 : it;
    if (out)
        *out = o;

    free(contrib); free(next_f); free(next_u); free(cfx);
    free(wl_curr); free(wl_next); free(resid);
    return 0;
}

/* Data-driven push (mode 7) and pull-push (mode 8) in the synchronous
 * order: every worklist vertex takes the residual it held when the
 * iteration began, and pull-push reads the ranks of that moment; pushes go
 * to the residuals in vertex order (which fixes the activation tests).  The
 * reference's OpenMP loop (pageRank.c:3049-3090) lies between this order
 * and the sequential one of orc_pagerank, as does a GPU run of the same
 * loop, whose vertices take their residuals with atomic exchanges at any
 * point of the iteration.  ranks: V floats out, divided by V. */
void orc_pagerank_dd_sync(const orc_csr *g, int mode, uint32_t iterations, double epsilon, float *ranks)
{
    const uint32_t V = g->V;
    const float damp = 0.85f, base = 1.0f - damp;
    float *resid = (float *)calloc((size_t)V + 1, sizeof(float));
    float *taken = (float *)calloc((size_t)V + 1, sizeof(float));
    float *old_rank = (float *)calloc((size_t)V + 1, sizeof(float));
    uint8_t *wl_curr = (uint8_t *)calloc((size_t)V + 1, 1);
    uint8_t *wl_next = (uint8_t *)calloc((size_t)V + 1, 1);
    for (uint32_t v = 0; v < V; v++)
    {
        ranks[v] = base;
        float r = 0.0f;
        for (uint32_t j = g->in_off[v]; j < g->in_off[v + 1]; j++)
        {
            uint32_t du = out_degree(g, g->in_adj[j]);
            if (du)
                r += 1.0f / (float)du;
        }
        resid[v] = (1.0f - damp) * damp * r;
        wl_curr[v] = 1;
    }
    for (uint32_t it = 0; it < iterations; it++)
    {
        uint32_t active = 0;
        for (uint32_t v = 0; v < V; v++)
        {
            old_rank[v] = ranks[v];
            taken[v] = 0.0f;
            if (wl_curr[v])
            {
                taken[v] = resid[v];
                resid[v] = 0.0f;
            }
        }
        for (uint32_t v = 0; v < V; v++)
        {
            if (!wl_curr[v])
                continue;
            if (mode == 7)
                ranks[v] = taken[v] + old_rank[v];
            else
            {
                float in_pr = 0.0f;
                for (uint32_t j = g->in_off[v]; j < g->in_off[v + 1]; j++)
                {
                    uint32_t u = g->in_adj[j];
                    in_pr += old_rank[u] / (float)out_degree(g, u);
                }
                ranks[v] = base + (damp * in_pr);
            }
            uint32_t deg = out_degree(g, v);
            float delta = damp * (taken[v] / deg);
            for (uint32_t j = g->out_off[v]; j < g->out_off[v + 1]; j++)
            {
                uint32_t u = g->out_adj[j];
                float prev = resid[u];
                resid[u] += delta;
                if ((fabs(prev + delta) >= epsilon) && (prev <= epsilon))
                {
                    active++;
                    if (mode == 8)
                        resid[u] += delta;
                    wl_next[u] = 1;
                }
            }
        }
        uint8_t *t = wl_curr; wl_curr = wl_next; wl_next = t;
        memset(wl_next, 0, V);
        if (active == 0)
            break;
    }
    for (uint32_t v = 0; v < V; v++)
        ranks[v] = ranks[v] / (float)V;
    free(resid); free(taken); free(old_rank); free(wl_curr); free(wl_next);
}

void orc_pagerank_f64(const orc_csr *g, uint32_t executed, int init_one_over_n, double *ranks)
{
    const uint32_t V = g->V;
    const double damp = 0.85, base = init_one_over_n ? 0.15 / V : 0.15;
    double *contrib = (double *)malloc(((size_t)V + 1) * sizeof(double));
    for (uint32_t v = 0; v < V; v++)
        ranks[v] = init_one_over_n ? 1.0 / V : 0.15;
    /* per-vertex sums run in CSC order whatever the thread count */
    for (uint32_t it = 0; it < executed; it++)
    {
#pragma omp parallel for schedule(static)
        for (uint32_t v = 0; v < V; v++)
        {
            uint32_t d = out_degree(g, v);
            contrib[v] = d ? ranks[v] / d : 0.0;
        }
#pragma omp parallel for schedule(dynamic, 1024)
        for (uint32_t v = 0; v < V; v++)
        {
            double s = 0.0;
            for (uint32_t j = g->in_off[v]; j < g->in_off[v + 1]; j++)
                s += contrib[g->in_adj[j]];
            ranks[v] = base + damp * s;
        }
    }
    if (!init_one_over_n)
        for (uint32_t v = 0; v < V; v++)
            ranks[v] /= V;
    free(contrib);
}

/* Personalised PageRank with a seed set S (seeds[0..nseeds), repeats
 * allowed): the reference's pull iteration (pageRank.c:1026-1069, no
 * dangling redistribution) with the uniform teleport replaced by one to the
 * seeds, each occurrence carrying 1/|S|:
 *   rank_0(v) = c(v)/|S|,  rank'(v) = (1-d) c(v)/|S| + d * sum_{u in in(v)} rank(u)/outdeg(u)
 * where c(v) counts v in S.  All in FP64, in-edges in CSC order. */
void orc_ppr_f64_multi(const orc_csr *g, const uint32_t *seeds, uint32_t nseeds, uint32_t iterations, double damp,
                       double *ranks)
{
    const uint32_t V = g->V;
    double *contrib = (double *)malloc(((size_t)V + 1) * sizeof(double));
    double *tele = (double *)calloc((size_t)V + 1, sizeof(double));
    for (uint32_t i = 0; i < nseeds; i++) tele[seeds[i]] += 1.0 / (double)nseeds;
    for (uint32_t v = 0; v < V; v++) ranks[v] = tele[v];
    /* per-vertex sums run in CSC order whatever the thread count */
    for (uint32_t it = 0; it < iterations; it++)
    {
#pragma omp parallel for schedule(static)
        for (uint32_t v = 0; v < V; v++)
        {
            uint32_t d = out_degree(g, v);
            contrib[v] = d ? ranks[v] / d : 0.0;
        }
#pragma omp parallel for schedule(dynamic, 1024)
        for (uint32_t v = 0; v < V; v++)
        {
            double s = 0.0;
            for (uint32_t j = g->in_off[v]; j < g->in_off[v + 1]; j++)
                s += contrib[g->in_adj[j]];
            ranks[v] = (1.0 - damp) * tele[v] + damp * s;
        }
    }
    free(tele);
    free(contrib);
}

void orc_ppr_f64(const orc_csr *g, uint32_t seed, uint32_t iterations, double damp, double *ranks)
{
    orc_ppr_f64_multi(g, &seed, 1, iterations, damp, ranks);
}

/* K personalised PageRank vectors advanced together, FP32, the CPU timing
 * baseline of the batched GPU form: ranks and contributions vertex-major
 * ([V][K], one row of K values per vertex, so every in-edge reads one
 * contiguous row), the per-vector arithmetic of orc_ppr_f64_multi in float
 * (contribution = rank / outdeg, rank' = tele + damp * sum).  init[v*K + k]
 * is vector k's starting rank (c_k(v)/|S_k|); the teleport is
 * (1 - damp) * init.  OpenMP over destination vertices, nthreads threads
 * (0: all). */
void orc_ppr_f32_batch(const orc_csr *g, uint32_t K, const float *init, uint32_t iterations, float damp,
                       int nthreads, float *ranks)
{
    const uint32_t V = g->V;
    if (nthreads <= 0) nthreads = omp_get_max_threads();
    float *contrib = (float *)malloc(((size_t)V * K + 1) * sizeof(float));
    float *tele = (float *)malloc(((size_t)V * K + 1) * sizeof(float));
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (uint32_t v = 0; v < V; v++)
        for (uint32_t k = 0; k < K; k++)
        {
            const size_t i = (size_t)v * K + k;
            tele[i] = (1.0f - damp) * init[i];
            ranks[i] = init[i];
        }
    for (uint32_t it = 0; it < iterations; it++)
    {
#pragma omp parallel for schedule(static) num_threads(nthreads)
        for (uint32_t v = 0; v < V; v++)
        {
            const uint32_t d = out_degree(g, v);
            const float fd = (float)d;
            for (uint32_t k = 0; k < K; k++)
                contrib[(size_t)v * K + k] = d ? ranks[(size_t)v * K + k] / fd : 0.0f;
        }
#pragma omp parallel num_threads(nthreads)
        {
            float *s = (float *)malloc((size_t)K * sizeof(float));
#pragma omp for schedule(dynamic, 1024)
            for (uint32_t v = 0; v < V; v++)
            {
                for (uint32_t k = 0; k < K; k++) s[k] = 0.0f;
                for (uint32_t j = g->in_off[v]; j < g->in_off[v + 1]; j++)
                {
                    const float *row = contrib + (size_t)g->in_adj[j] * K;
                    for (uint32_t k = 0; k < K; k++) s[k] += row[k];
                }
                for (uint32_t k = 0; k < K; k++)
                    ranks[(size_t)v * K + k] = tele[(size_t)v * K + k] + damp * s[k];
            }
            free(s);
        }
    }
    free(tele);
    free(contrib);
}

/* ------------------------------------------------------------------------ */
/* BFS                                                                       */
/* ------------------------------------------------------------------------ */

typedef struct bfs_state
{
    const orc_csr *g;
    int32_t *parents;
    uint32_t *distances;
    uint64_t edges;
    int nthreads;
} bfs_state;

static inline int bit_get(const uint32_t *bm, uint32_t v) { return (bm[v >> 5] >> (v & 31)) & 1u; }

/* topDownStepGraphCSR (BFS.c:688-750): CAS claim of unvisited out-neighbours.
 * Returns mf and writes the next frontier queue. */
static uint32_t td_step_queue(bfs_state *s, const uint32_t *q, uint32_t qn, uint32_t *nq, uint32_t *nqn,
                              uint32_t *nbm)
{
    const orc_csr *g = s->g;
    uint32_t mf = 0;
    uint32_t count = 0;
    uint64_t edges = 0;
#pragma omp parallel num_threads(s->nthreads) reduction(+ : mf, edges)
    {
        uint32_t *local = NULL;
        uint32_t ln = 0, lcap = 0;
#pragma omp for schedule(dynamic, 64)
        for (uint32_t i = 0; i < qn; i++)
        {
            uint32_t v = q[i];
            for (uint32_t j = g->out_off[v]; j < g->out_off[v + 1]; j++)
            {
                uint32_t u = g->out_adj[j];
                int32_t up = s->parents[u];
                edges++;
                if (up < 0)
                {
                    if (__sync_bool_compare_and_swap(&s->parents[u], up, (int32_t)v))
                    {
                        if (ln == lcap)
                        {
                            lcap = lcap ? lcap * 2 : 1024;
                            local = (uint32_t *)realloc(local, (size_t)lcap * sizeof(uint32_t));
                        }
                        local[ln++] = u;
                        mf += (uint32_t)(-up);
                        s->distances[u] = s->distances[v] + 1;
                    }
                }
            }
        }
        if (ln)
        {
            uint32_t at = __sync_fetch_and_add(&count, ln);
            if (nq)
                memcpy(nq + at, local, (size_t)ln * sizeof(uint32_t));
            if (nbm)
                for (uint32_t k = 0; k < ln; k++)
                    __sync_fetch_and_or(&nbm[local[k] >> 5], 1u << (local[k] & 31));
        }
        free(local);
    }
    *nqn = count;
    s->edges += edges;
    return mf;
}

/* topDownStepUsingBitmapsGraphCSR (BFS.c:1062-1110): frontier as a bitmap,
 * scanned in vertex order. */
static uint32_t td_step_bitmap(bfs_state *s, const uint32_t *bm, uint32_t *nbm)
{
    const orc_csr *g = s->g;
    uint32_t mf = 0;
    uint64_t edges = 0;
#pragma omp parallel for schedule(dynamic, 1024) num_threads(s->nthreads) reduction(+ : mf, edges)
    for (uint32_t v = 0; v < g->V; v++)
    {
        if (!bit_get(bm, v))
            continue;
        for (uint32_t j = g->out_off[v]; j < g->out_off[v + 1]; j++)
        {
            uint32_t u = g->out_adj[j];
            int32_t up = s->parents[u];
            edges++;
            if (up < 0 && __sync_bool_compare_and_swap(&s->parents[u], up, (int32_t)v))
            {
                mf += (uint32_t)(-up);
                s->distances[u] = s->distances[v] + 1;
                __sync_fetch_and_or(&nbm[u >> 5], 1u << (u & 31));
            }
        }
    }
    s->edges += edges;
    return mf;
}

/* bottomUpStepGraphCSR (BFS.c:752-803): every unvisited vertex scans its
 * in-neighbours (inverse CSR under DIRECTED) and takes the first one in the
 * frontier.  write_dist = 0 is the FPGA variant (no distances, BFS.c:791). */
static uint32_t bu_step(bfs_state *s, const uint32_t *bm, uint32_t *nbm, int write_dist)
{
    const orc_csr *g = s->g;
    uint32_t nf = 0;
    uint64_t edges = 0;
#pragma omp parallel for schedule(dynamic, 1024) num_threads(s->nthreads) reduction(+ : nf, edges)
    for (uint32_t v = 0; v < g->V; v++)
    {
        if (s->parents[v] >= 0)
            continue;
        for (uint32_t j = g->in_off[v]; j < g->in_off[v + 1]; j++)
        {
            uint32_t u = g->in_adj[j];
            edges++;
            if (bit_get(bm, u))
            {
                s->parents[v] = (int32_t)u;
                if (write_dist)
                    s->distances[v] = s->distances[u] + 1;
                __sync_fetch_and_or(&nbm[v >> 5], 1u << (v & 31));
                nf++;
                break;
            }
        }
    }
    s->edges += edges;
    return nf;
}

static uint32_t popcount_bitmap(const uint32_t *bm, uint32_t words)
{
    uint32_t n = 0;
    for (uint32_t i = 0; i < words; i++)
        n += (uint32_t)__builtin_popcount(bm[i]);
    return n;
}

void orc_bfs(const orc_csr *g, int mode, int source, int32_t *parents, uint32_t *distances,
             orc_bfs_out *out, int nthreads)
{
    const uint32_t V = g->V;
    orc_bfs_out o = {0};
    /* newBFSStatsGraphCSR (BFS.c:45-81) */
    for (uint32_t v = 0; v < V; v++)
    {
        uint32_t d = out_degree(g, v);
        distances[v] = 0;
        parents[v] = d ? -(int32_t)d : -1;
    }
    /* source check (BFS.c:293-301): `source > num_vertices` compares as
     * unsigned; source == num_vertices reads past label_array in the
     * reference and is rejected here. */
    if ((uint32_t)source >= V)
    {
        if (out)
            *out = o;
        return;
    }
    o.valid_source = 1;
    o.processed_nodes = 1; /* ++stats->processed_nodes in the first row */
    const uint32_t src = (uint32_t)source; /* label_array is the identity */
    const uint32_t words = (V + 31) / 32;
    bfs_state s = {g, parents, distances, 0, nthreads < 1 ? 1 : nthreads};

    uint32_t *q = (uint32_t *)malloc(((size_t)V + 1) * sizeof(uint32_t));
    uint32_t *nq = (uint32_t *)malloc(((size_t)V + 1) * sizeof(uint32_t));
    uint32_t *bm = (uint32_t *)calloc(words + 1, sizeof(uint32_t));
    uint32_t *nbm = (uint32_t *)calloc(words + 1, sizeof(uint32_t));
    uint32_t qn = 0, nqn = 0;
    const uint32_t alpha = 15, beta = 18;

    parents[src] = (int32_t)src;

    if (mode == 0)
    {
        /* breadthFirstSearchPullGraphCSR (BFS.c:284-422): bottom-up every level */
        bm[src >> 5] |= 1u << (src & 31);
        uint32_t nf = 1;
        while (nf)
        {
            memset(nbm, 0, words * sizeof(uint32_t));
            nf = bu_step(&s, bm, nbm, 0);
            uint32_t *t = bm; bm = nbm; nbm = t;
            o.processed_nodes += nf;
            o.bottom_up_steps++;
        }
    }
    else if (mode == 1)
    {
        /* breadthFirstSearchPushGraphCSR (BFS.c:424-523) */
        q[0] = src; qn = 1;
        while (qn)
        {
            td_step_queue(&s, q, qn, nq, &nqn, NULL);
            uint32_t *t = q; q = nq; nq = t;
            qn = nqn;
            o.processed_nodes += qn;
            o.top_down_steps++;
        }
    }
    else if (mode == 3)
    {
        /* breadthFirstSearchPushBitmapGraphCSR (BFS.c:841-930) */
        bm[src >> 5] |= 1u << (src & 31);
        uint32_t n = 1;
        while (n)
        {
            memset(nbm, 0, words * sizeof(uint32_t));
            td_step_bitmap(&s, bm, nbm);
            uint32_t *t = bm; bm = nbm; nbm = t;
            n = popcount_bitmap(bm, words);
            o.processed_nodes += n;
            o.top_down_steps++;
        }
    }
    else if (mode == 4)
    {
        /* breadthFirstSearchPushDirectionOptimizedBitmapGraphCSR (BFS.c:932-1060) */
        uint32_t mu = g->E, mf = out_degree(g, src), nf = 0, nf_prev = 0, n = V;
        bm[src >> 5] |= 1u << (src & 31);
        uint32_t bits = 1;
        while (bits)
        {
            if (mf > (mu / alpha))
            {
                nf = bits;
                do
                {
                    nf_prev = nf;
                    memset(nbm, 0, words * sizeof(uint32_t));
                    nf = bu_step(&s, bm, nbm, 1);
                    uint32_t *t = bm; bm = nbm; nbm = t;
                    bits = nf;
                    o.processed_nodes += nf;
                    o.bottom_up_steps++;
                } while ((nf > nf_prev) || (nf > (n / beta)));
                mf = 1;
            }
            else
            {
                mu -= mf;
                memset(nbm, 0, words * sizeof(uint32_t));
                mf = td_step_bitmap(&s, bm, nbm);
                uint32_t *t = bm; bm = nbm; nbm = t;
                bits = popcount_bitmap(bm, words);
                o.processed_nodes += bits;
                o.top_down_steps++;
            }
        }
    }
    else
    {
        /* breadthFirstSearchDirectionOptimizedGraphCSR (BFS.c:525-686), also
         * the dispatcher's default (BFS.c:263-265) */
        uint32_t mu = g->E, mf = out_degree(g, src), nf = 0, nf_prev = 0, n = V;
        q[0] = src; qn = 1;
        while (qn)
        {
            if (mf > (mu / alpha))
            {
                memset(bm, 0, words * sizeof(uint32_t));
                for (uint32_t i = 0; i < qn; i++)
                    bm[q[i] >> 5] |= 1u << (q[i] & 31);
                nf = qn;
                do
                {
                    nf_prev = nf;
                    memset(nbm, 0, words * sizeof(uint32_t));
                    nf = bu_step(&s, bm, nbm, 1);
                    uint32_t *t = bm; bm = nbm; nbm = t;
                    o.processed_nodes += nf;
                    o.bottom_up_steps++;
                } while ((nf > nf_prev) || (nf > (n / beta)));
                /* bitmapToArrayQueue: ascending vertex order */
                qn = 0;
                for (uint32_t v = 0; v < V; v++)
                    if (bit_get(bm, v))
                        q[qn++] = v;
                mf = 1;
            }
            else
            {
                mu -= mf;
                mf = td_step_queue(&s, q, qn, nq, &nqn, NULL);
                uint32_t *t = q; q = nq; nq = t;
                qn = nqn;
                o.processed_nodes += qn;
                o.top_down_steps++;
            }
        }
    }
    o.edges_examined = s.edges;
    o.iteration = 1 + o.top_down_steps + o.bottom_up_steps;
    if (out)
        *out = o;
    free(q); free(nq); free(bm); free(nbm);
}

/* ------------------------------------------------------------------------ */
/* SpMV                                                                      */
/* ------------------------------------------------------------------------ */

static double checksum_round2(const float *y, uint32_t V)
{
    /* SPMV.c:727-730: sum += ((int)(y * 100 + .5) / 100.0) */
    double sum = 0.0;
    for (uint32_t v = 0; v < V; v++)
        sum += ((int)(y[v] * 100 + .5) / 100.0);
    return sum;
}

int orc_spmv(const orc_csr *g, int mode, uint32_t iterations, const float *x_in,
             float *x_out, float *y, double *checksum, int nthreads)
{
    const uint32_t V = g->V;
    if (mode < 0 || mode > 3)
        return -1;
#ifndef _OPENMP
    (void)nthreads;
#else
    if (nthreads < 1)
        nthreads = 1;
#endif
    /* input vector (SPMV.c:696-701) */
    for (uint32_t v = 0; v < V; v++)
    {
        if (x_in)
            x_out[v] = x_in[v];
        else
        {
            uint32_t d = out_degree(g, v);
            x_out[v] = d ? (1.0f / d) : 0.001f;
        }
        y[v] = 0.0f;
    }
    const float *x = x_out;

    if (mode == 0)
    {
        /* pull: the SpMV CU's sum (cu_SPMV/CSR/PULL/FloatPoint) over in-edges */
        for (uint32_t it = 0; it < iterations; it++)
        {
#pragma omp parallel for schedule(dynamic, 1024) num_threads(nthreads)
            for (uint32_t v = 0; v < V; v++)
            {
                float s = 0.0f;
                for (uint32_t j = g->in_off[v]; j < g->in_off[v + 1]; j++)
                {
                    float w = g->in_w ? g->in_w[j] : 0.0001f;
                    s += w * x[g->in_adj[j]];
                }
                y[v] = s;
            }
        }
    }
    else if (mode == 1)
    {
        /* push (SPMV.c:795-820): y accumulates across iterations */
        for (uint32_t it = 0; it < iterations; it++)
            for (uint32_t v = 0; v < V; v++)
                for (uint32_t j = g->out_off[v]; j < g->out_off[v + 1]; j++)
                {
                    float w = g->out_w ? g->out_w[j] : 0.0001f;
                    y[g->out_adj[j]] += (w * x[v]);
                }
    }
    else if (mode == 2)
    {
        /* pull fixed point: Q16.16 operands, product >> 16 accumulated in
         * 64 bits (cu_SPMV/CSR/PULL/FixedPoint/cu/cu_sum_kernel_control.sv:155-184,
         * SCALEF = 16 in its globals_cu_pkg.sv:37), y = Fixed32ToFloat(sum) */
        uint32_t *x32 = (uint32_t *)malloc(((size_t)V + 1) * sizeof(uint32_t));
        for (uint32_t v = 0; v < V; v++)
            x32[v] = orc_fx32_from_float(x[v]);
        for (uint32_t it = 0; it < iterations; it++)
            for (uint32_t v = 0; v < V; v++)
            {
                uint64_t s = 0;
                for (uint32_t j = g->in_off[v]; j < g->in_off[v + 1]; j++)
                {
                    uint32_t w32 = orc_fx32_from_float(g->in_w ? g->in_w[j] : 0.0001f);
                    s += ((uint64_t)x32[g->in_adj[j]] * (uint64_t)w32) >> 16;
                }
                y[v] = orc_fx32_to_float(s);
            }
        free(x32);
    }
    else
    {
        /* push fixed point (SPMV.c:1017-1135): Q32.32, y64 += (w*x) >> 32 */
        uint64_t *x64 = (uint64_t *)malloc(((size_t)V + 1) * sizeof(uint64_t));
        uint64_t *y64 = (uint64_t *)calloc((size_t)V + 1, sizeof(uint64_t));
        for (uint32_t v = 0; v < V; v++)
            x64[v] = orc_fx64_from_double(x[v]);
        for (uint32_t it = 0; it < iterations; it++)
            for (uint32_t v = 0; v < V; v++)
                for (uint32_t j = g->out_off[v]; j < g->out_off[v + 1]; j++)
                {
                    uint64_t w64 = orc_fx64_from_double(g->out_w ? g->out_w[j] : 0.0001f);
                    y64[g->out_adj[j]] += orc_fx64_mul(w64, x64[v]);
                }
        for (uint32_t v = 0; v < V; v++)
            y[v] = (float)orc_fx64_to_double(y64[v]);
        free(x64);
        free(y64);
    }
    if (checksum)
        *checksum = checksum_round2(y, V);
    return 0;
}

void orc_spmv_f64(const orc_csr *g, const float *x, double *y)
{
#pragma omp parallel for schedule(dynamic, 1024)
    for (uint32_t v = 0; v < g->V; v++)
    {
        double s = 0.0;
        for (uint32_t j = g->in_off[v]; j < g->in_off[v + 1]; j++)
        {
            double w = g->in_w ? (double)g->in_w[j] : (double)0.0001f;
            s += w * (double)x[g->in_adj[j]];
        }
        y[v] = s;
    }
}

/* ------------------------------------------------------------------------ */
/* connected components                                                      */
/* ------------------------------------------------------------------------ */

static uint32_t uf_find(uint32_t *p, uint32_t x)
{
    while (p[x] != x)
    {
        p[x] = p[p[x]];
        x = p[x];
    }
    return x;
}

void orc_cc_min_label(const orc_csr *g, uint32_t *comp)
{
    const uint32_t V = g->V;
    for (uint32_t v = 0; v < V; v++)
        comp[v] = v;
    for (uint32_t u = 0; u < V; u++)
        for (uint32_t j = g->out_off[u]; j < g->out_off[u + 1]; j++)
        {
            uint32_t a = uf_find(comp, u), b = uf_find(comp, g->out_adj[j]);
            if (a == b)
                continue;
            /* the smaller id stays the root */
            if (a < b)
                comp[b] = a;
            else
                comp[a] = b;
        }
    for (uint32_t v = 0; v < V; v++)
        comp[v] = uf_find(comp, v);
}

static void cc_compress(uint32_t V, uint32_t *comp)
{
    for (uint32_t n = 0; n < V; n++)
        while (comp[n] != comp[comp[n]])
            comp[n] = comp[comp[n]];
}

uint32_t orc_cc_sv(const orc_csr *g, uint32_t *comp)
{
    const uint32_t V = g->V;
    for (uint32_t v = 0; v < V; v++)
        comp[v] = v;
    uint32_t iterations = 0, change = 1;
    while (change)
    {
        change = 0;
        iterations++;
        for (uint32_t u = 0; u < V; u++)
            for (uint32_t j = g->out_off[u]; j < g->out_off[u + 1]; j++)
            {
                const uint32_t cu = comp[u], cv = comp[g->out_adj[j]];
                if (cu == cv)
                    continue;
                const uint32_t high = cu > cv ? cu : cv, low = cu > cv ? cv : cu;
                if (comp[high] == high)
                {
                    comp[high] = low;
                    change = 1;
                }
            }
        cc_compress(V, comp);
    }
    return iterations;
}

/* union of the trees of u and v, the lower label becoming the parent
 * (compare-and-swap on a root; retried while the roots move) */
static void cc_link(uint32_t u, uint32_t v, uint32_t *comp)
{
    uint32_t a = comp[u], b = comp[v];
    while (a != b)
    {
        const uint32_t hi = a > b ? a : b, lo = a > b ? b : a;
        const uint32_t ph = comp[hi];
        if (ph == lo)
            break;
        if (ph == hi && __sync_bool_compare_and_swap(&comp[hi], hi, lo))
            break;
        a = comp[comp[hi]];
        b = comp[lo];
    }
}

static void cc_compress_par(uint32_t V, uint32_t *comp, int nthreads)
{
#pragma omp parallel for schedule(dynamic, 2048) num_threads(nthreads)
    for (uint32_t n = 0; n < V; n++)
        while (comp[n] != comp[comp[n]])
            comp[n] = comp[comp[n]];
}

void orc_cc_afforest(const orc_csr *g, uint32_t rounds, uint32_t samples, uint64_t seed, int use_in,
                     uint32_t *comp, int nthreads)
{
    const uint32_t V = g->V;
    for (uint32_t v = 0; v < V; v++)
        comp[v] = v;
    for (uint32_t r = 0; r < rounds; r++)
    {
#pragma omp parallel for schedule(dynamic, 2048) num_threads(nthreads)
        for (uint32_t u = 0; u < V; u++)
            if (g->out_off[u] + r < g->out_off[u + 1])
                cc_link(u, g->out_adj[g->out_off[u] + r], comp);
        cc_compress_par(V, comp, nthreads);
    }
    /* the most frequent label among `samples` vertices */
    uint32_t skip = 0xffffffffu;
    if (V && samples)
    {
        uint32_t *s = (uint32_t *)malloc((size_t)samples * 4);
        for (uint32_t i = 0; i < samples; i++)
            s[i] = comp[orc_splitmix64(seed + i) % V];
        uint32_t best = 0;
        for (uint32_t i = 0; i < samples; i++)
        {
            uint32_t c = 0;
            for (uint32_t k = 0; k < samples; k++)
                c += s[k] == s[i];
            if (c > best || (c == best && s[i] < skip))
            {
                best = c;
                skip = s[i];
            }
        }
        free(s);
    }
#pragma omp parallel for schedule(dynamic, 2048) num_threads(nthreads)
    for (uint32_t u = 0; u < V; u++)
    {
        if (comp[u] == skip)
            continue;
        for (uint32_t j = g->out_off[u] + rounds; j < g->out_off[u + 1]; j++)
            cc_link(u, g->out_adj[j], comp);
        if (use_in)
            for (uint32_t j = g->in_off[u]; j < g->in_off[u + 1]; j++)
                cc_link(u, g->in_adj[j], comp);
    }
    cc_compress_par(V, comp, nthreads);
}
