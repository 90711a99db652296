/*
 * Autotuner for the launch shapes of the hot kernels (no counterpart in the
 * reference, whose one run-time knob of this kind is the work granularity
 * binSize, 02_capi_graph/include/config/graphConfig.h:18).
 *
 * gg_autotune times candidate shapes on the caller's mapping and keeps the
 * fastest on it; the pick is also remembered for the graph's class, so a
 * later mapping of a graph of the same class on a GPU with the same SM count
 * starts with it (gg_tune_lookup, on its first call), and the remembered
 * picks can be saved to a text file and loaded in another process.
 *
 * Families and their search spaces (the default shape is always one of the
 * candidates, so a pick is never slower than the default on the timings it
 * was chosen from):
 *   PR, SPMV  the FP pull gather of PageRank / SpMV: the hot-vertex table off
 *             with 3, 4, 5, 6 or 8 resident CTAs per SM, or on with one CTA
 *             of 16, 24 or 32 warps per SM; measured: mean device time of a
 *             gather launch (profile events);
 *   BFS       the top-down heavy-vertex threshold (32, 64, 128, 256, 1024
 *             out-edges) of the direction-optimising search; measured: device
 *             time of eight searches from fixed sources;
 *   PPR       merge items per tile of the batched personalised PageRank
 *             (256, 512, 1024); measured: one K = 64 run of 5 iterations;
 *   BATCH     (runs without an epsilon stop) the union pull against the
 *             many-graphs kernel, and the
 *             kernel's shape: resident CTAs per SM x warps per CTA (2 x 16,
 *             1 x 32, 1 x 16, 2 x 8, 4 x 8, 8 x 4), then the bin threshold (0, 1024,
 *             4096, 8192 vertices in shared memory), then items per lane (5,
 *             7, 9), each stage keeping the best of the one before
 *             (coordinate descent); measured: one run of the batch.
 * Every candidate runs once untimed, then `reps` timed runs; the median
 * decides.
 *
 * Graph class: floor(log2 V), round(log2(E / V)), round(log2(max out-degree
 * / mean out-degree)), the storage format and the SM count; for BATCH the
 * class adds floor(log2 ngraphs).
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "gg_internal.h"

namespace {

struct Key
{
    uint32_t family, storage, vlog, dlog, slog, sms, glog;
    bool operator<(const Key &o) const
    {
        return std::tie(family, storage, vlog, dlog, slog, sms, glog) <
               std::tie(o.family, o.storage, o.vlog, o.dlog, o.slog, o.sms, o.glog);
    }
};

struct Pick
{
    uint32_t v[5];
};

std::mutex g_mu;
std::map<Key, Pick> g_cache;

__global__ void k_max_u32(const uint32_t *__restrict__ x, uint32_t n, uint32_t *out)
{
    uint32_t m = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) m = max(m, x[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}

uint32_t ilog2(double x) { return x >= 1.0 ? (uint32_t)floor(log2(x)) : 0u; }
uint32_t rlog2(double x) { return x >= 1.0 ? (uint32_t)lround(log2(x)) : 0u; }

/* the class of g (family and storage filled in by the caller) */
gg_status graph_class(gg_graph *g, cudaStream_t s, Key &k)
{
    uint32_t *d = nullptr, *h = nullptr;
    void *p;
    GG_CHECK(gg_work(g, 27, 16, &p));
    d = (uint32_t *)p;
    GG_CHECK(gg_pinned(g, 64, (void **)&h));
    GG_CUDA(cudaMemsetAsync(d, 0, 4, s));
    if (g->V) k_max_u32<<<gg_sm_count() * 4, 256, 0, s>>>(g->out_deg, g->V, d);
    GG_CUDA(cudaGetLastError());
    GG_CUDA(cudaMemcpyAsync(h, d, 4, cudaMemcpyDeviceToHost, s));
    GG_CHECK(gg_wait(s));
    const double avg = g->V ? (double)g->E / (double)g->V : 0.0;
    k.vlog = ilog2((double)g->V);
    k.dlog = rlog2(avg);
    k.slog = avg > 0.0 ? rlog2((double)h[0] / avg) : 0u;
    k.sms = (uint32_t)gg_sm_count();
    k.glog = 0;
    return GG_OK;
}

void remember(const Key &k, const Pick &p)
{
    std::lock_guard<std::mutex> lk(g_mu);
    g_cache[k] = p;
}

bool recall(const Key &k, Pick &p)
{
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_cache.find(k);
    if (it == g_cache.end()) return false;
    p = it->second;
    return true;
}

float median(std::vector<float> v)
{
    if (v.empty()) return INFINITY;
    std::sort(v.begin(), v.end());
    return v[v.size() / 2];
}

/* time `run` (which queues work on s and returns a status): one untimed
 * run, then reps runs between events; the median device time */
template <class F>
gg_status time_runs(gg_graph *g, cudaStream_t s, uint32_t reps, F run, float *ms)
{
    GG_CHECK(run());
    std::vector<float> t;
    cudaEvent_t a, b;
    GG_CHECK(gg_event_at(g, 60, &a));
    GG_CHECK(gg_event_at(g, 61, &b));
    for (uint32_t i = 0; i < reps; i++)
    {
        GG_CUDA(cudaEventRecord(a, s));
        GG_CHECK(run());
        GG_CUDA(cudaEventRecord(b, s));
        GG_CHECK(gg_wait(s));
        t.push_back(gg_event_ms(a, b));
    }
    *ms = median(t);
    return GG_OK;
}

gg_status tune_pull(gg_graph *g, bool spmv, uint32_t storage, uint32_t reps, cudaStream_t s, gg_tune_choice &c)
{
    const gg_pull_shape keep = spmv ? g->spmv_shape : g->pr_shape;
    std::vector<gg_pull_shape> cands;
    gg_pull_shape dflt;
    cands.push_back(dflt);
    for (uint32_t ctas : {3u, 4u, 5u, 6u, 8u})
    {
        gg_pull_shape x;
        x.hot = 0;
        x.ctas = ctas;
        cands.push_back(x);
    }
    if (g->V < GG_HOT_FLAG)
        for (uint32_t w : {16u, 24u, 32u})
        {
            gg_pull_shape x;
            x.hot = 1;
            x.hot_warps = w;
            cands.push_back(x);
        }
    float best = INFINITY;
    gg_pull_shape pick = dflt;
    for (size_t i = 0; i < cands.size(); i++)
    {
        (spmv ? g->spmv_shape : g->pr_shape) = cands[i];
        float ms = INFINITY;
        gg_status st;
        if (spmv)
        {
            gg_spmv_params p = {GG_SPMV_PULL, storage, 3, 1, 0};
            std::vector<float> t;
            st = GG_OK;
            for (uint32_t r = 0; r <= reps && st == GG_OK; r++)
            {
                gg_spmv_result res;
                st = gg_spmv(g, &p, nullptr, nullptr, nullptr, &res, s);
                if (st == GG_OK && r > 0) t.push_back(res.spmv_ms / (float)std::max(res.spmv_launches, 1u));
            }
            ms = median(t);
        }
        else
        {
            gg_pr_params p = {GG_PR_PULL, storage, 3, 0, 0.0, 0.85f, 1, 0};
            std::vector<float> t;
            st = GG_OK;
            for (uint32_t r = 0; r <= reps && st == GG_OK; r++)
            {
                gg_pr_result res;
                st = gg_pagerank(g, &p, nullptr, &res, s);
                if (st == GG_OK && r > 0) t.push_back(res.gather_ms / (float)std::max(res.gather_launches, 1u));
            }
            ms = median(t);
        }
        if (st != GG_OK)
        {
            (spmv ? g->spmv_shape : g->pr_shape) = keep;
            return st;
        }
        if (i == 0) c.default_ms = ms;
        if (ms < best)
        {
            best = ms;
            pick = cands[i];
        }
    }
    (spmv ? g->spmv_shape : g->pr_shape) = pick;
    g->tuned |= spmv ? GG_TUNE_SPMV : GG_TUNE_PR;
    c.family = spmv ? GG_TUNE_SPMV : GG_TUNE_PR;
    c.params[0] = pick.hot;
    c.params[1] = pick.ctas;
    c.params[2] = pick.hot_warps;
    c.tuned_ms = best;
    c.candidates = (uint32_t)cands.size();
    return GG_OK;
}

gg_status tune_bfs(gg_graph *g, uint32_t reps, cudaStream_t s, gg_tune_choice &c)
{
    /* eight sources with out-edges, spread over the id range */
    std::vector<uint32_t> deg(g->V);
    GG_CHECK(gg_wait(s));
    GG_CUDA(cudaMemcpy(deg.data(), g->out_deg, (size_t)g->V * 4, cudaMemcpyDeviceToHost));
    std::vector<uint32_t> src;
    for (uint32_t k = 0; k < 8; k++)
    {
        uint32_t v = (uint32_t)(((uint64_t)g->V * (2 * k + 1)) / 16);
        for (uint32_t n = 0; n < g->V && deg[v] == 0; n++) v = v + 1 < g->V ? v + 1 : 0;
        if (deg[v]) src.push_back(v);
    }
    if (src.empty()) return GG_OK;
    const uint32_t keep = g->bfs_heavy;
    float best = INFINITY;
    uint32_t pick = 64;
    uint32_t n = 0;
    for (uint32_t thr : {64u, 32u, 128u, 256u, 1024u})
    {
        g->bfs_heavy = thr;
        float ms = INFINITY;
        gg_status st = time_runs(g, s, reps, [&]() -> gg_status {
            for (uint32_t v : src)
            {
                gg_bfs_params p = {GG_BFS_DO, v, 15, 18, 0};
                gg_bfs_result r;
                GG_CHECK(gg_bfs(g, &p, nullptr, nullptr, &r, s));
            }
            return GG_OK;
        }, &ms);
        if (st != GG_OK)
        {
            g->bfs_heavy = keep;
            return st;
        }
        if (n++ == 0) c.default_ms = ms;
        if (ms < best)
        {
            best = ms;
            pick = thr;
        }
    }
    g->bfs_heavy = pick;
    c.family = GG_TUNE_BFS;
    c.params[0] = pick;
    c.tuned_ms = best;
    c.candidates = n;
    return GG_OK;
}

gg_status tune_ppr(gg_graph *g, uint32_t storage, uint32_t reps, cudaStream_t s, gg_tune_choice &c)
{
    std::vector<uint32_t> deg(g->V);
    GG_CHECK(gg_wait(s));
    GG_CUDA(cudaMemcpy(deg.data(), g->out_deg, (size_t)g->V * 4, cudaMemcpyDeviceToHost));
    std::vector<uint32_t> seeds, off(1, 0);
    for (uint32_t v = 0; v < g->V && seeds.size() < 64; v += std::max(1u, g->V / 64))
        if (deg[v])
        {
            seeds.push_back(v);
            off.push_back((uint32_t)seeds.size());
        }
    if (seeds.empty()) return GG_OK;
    const uint32_t K = (uint32_t)seeds.size();
    const uint32_t keep = g->ppr_tile;
    float best = INFINITY;
    uint32_t pick = 512, n = 0;
    for (uint32_t tile : {512u, 256u, 1024u})
    {
        g->ppr_tile = tile;
        float ms = INFINITY;
        gg_ppr_params p = {K, 5, 0.85f, (uint32_t)(storage == GG_STORE_F32 ? GG_STORE_F32 : GG_STORE_BF16), 0};
        gg_status st = time_runs(g, s, reps, [&]() -> gg_status {
            gg_ppr_result r;
            return gg_ppr(g, &p, off.data(), seeds.data(), nullptr, &r, s);
        }, &ms);
        if (st != GG_OK)
        {
            g->ppr_tile = keep;
            return st;
        }
        if (n++ == 0) c.default_ms = ms;
        if (ms < best)
        {
            best = ms;
            pick = tile;
        }
    }
    g->ppr_tile = pick;
    c.family = GG_TUNE_PPR;
    c.params[0] = pick;
    c.tuned_ms = best;
    c.candidates = n;
    return GG_OK;
}

gg_status tune_batch(gg_graph *g, uint32_t ngraphs, const uint32_t *voff, uint32_t reps, cudaStream_t s,
                     gg_tune_choice &c)
{
    const gg_graphs_config keep = g->graphs_cfg;
    const uint32_t tuned_before = g->tuned;
    float best = INFINITY;
    uint32_t n = 0;
    gg_pr_params p = {GG_PR_PULL, GG_STORE_F32, 20, 0, 0.0, 0.85f, 0, 0};
    auto run_cfg = [&](const gg_graphs_config &x, float *ms) -> gg_status {
        *ms = INFINITY;
        if (x.strategy == 1 && gg_pagerank_batch_config(g, x.ipt, x.warps, x.smem_vmax, x.ctas) != GG_OK)
        {
            gg_last_error();
            return GG_OK; /* does not fit */
        }
        g->graphs_cfg.strategy = x.strategy;
        return time_runs(g, s, reps, [&]() -> gg_status {
            gg_pr_result r;
            return gg_pagerank_batch(g, &p, ngraphs, voff, nullptr, &r, s);
        }, ms);
    };
    gg_graphs_config bestc;
    auto consider = [&](const gg_graphs_config &x) -> gg_status {
        float ms;
        GG_CHECK(run_cfg(x, &ms));
        if (n++ == 0) c.default_ms = ms;
        if (ms < best)
        {
            best = ms;
            bestc = x;
        }
        return GG_OK;
    };
    /* the default first: the union pull; then the kernel's default shape */
    gg_graphs_config dflt;
    dflt.strategy = 2;
    gg_status st = consider(dflt);
    gg_graphs_config other = dflt;
    other.strategy = 1;
    if (st == GG_OK) st = consider(other);
    /* the kernel's shape: CTAs x warps, then the bin, then items per lane */
    gg_graphs_config base;
    base.strategy = 1;
    const uint32_t shapes[][2] = {{2, 16}, {1, 32}, {1, 16}, {2, 8}, {4, 8}, {8, 4}};
    gg_graphs_config kbest = base;
    float kms = INFINITY;
    auto stage = [&](const gg_graphs_config &x) -> gg_status {
        float ms;
        GG_CHECK(run_cfg(x, &ms));
        n++;
        if (ms < kms)
        {
            kms = ms;
            kbest = x;
        }
        if (ms < best)
        {
            best = ms;
            bestc = x;
        }
        return GG_OK;
    };
    for (const auto &sh : shapes)
    {
        if (st != GG_OK) break;
        gg_graphs_config x = base;
        x.ctas = sh[0];
        x.warps = sh[1];
        st = stage(x);
    }
    const gg_graphs_config k1 = kbest;
    for (uint32_t vmax : {0u, 1024u, 8192u})
    {
        if (st != GG_OK) break;
        gg_graphs_config x = k1;
        x.smem_vmax = vmax;
        st = stage(x);
    }
    const gg_graphs_config k2 = kbest;
    for (uint32_t ipt : {5u, 9u})
    {
        if (st != GG_OK) break;
        gg_graphs_config x = k2;
        x.ipt = ipt;
        st = stage(x);
    }
    if (st != GG_OK)
    {
        g->graphs_cfg = keep;
        g->tuned = tuned_before;
        return st;
    }
    /* the kernel's best shape is kept even when the union pull wins */
    g->graphs_cfg = kbest;
    g->graphs_cfg.strategy = bestc.strategy;
    g->tuned |= GG_TUNE_BATCH;
    c.family = GG_TUNE_BATCH;
    c.params[0] = kbest.ipt;
    c.params[1] = kbest.warps;
    c.params[2] = kbest.smem_vmax;
    c.params[3] = kbest.ctas;
    c.params[4] = bestc.strategy;
    c.tuned_ms = best;
    c.candidates = n;
    return GG_OK;
}

} // namespace

gg_graphs_config gg_graphs_choice(gg_graph *g, uint32_t ngraphs)
{
    if (g->tuned & GG_TUNE_BATCH) return g->graphs_cfg;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (g_cache.empty()) return g->graphs_cfg;
    }
    Key k{};
    Pick p;
    if (graph_class(g, gg_stream(g, nullptr), k) != GG_OK) return g->graphs_cfg;
    k.family = GG_TUNE_BATCH;
    k.storage = 0;
    k.glog = ilog2((double)ngraphs);
    if (recall(k, p))
    {
        if (gg_pagerank_batch_config(g, p.v[0], p.v[1], p.v[2], p.v[3]) != GG_OK) gg_last_error();
        g->graphs_cfg.strategy = p.v[4];
    }
    return g->graphs_cfg;
}

void gg_tune_lookup(gg_graph *g, cudaStream_t s)
{
    if (g->tune_looked_up) return;
    g->tune_looked_up = true;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (g_cache.empty()) return;
    }
    Key k{};
    if (graph_class(g, s, k) != GG_OK) return;
    Pick p;
    k.storage = 0;
    k.family = GG_TUNE_PR;
    if (!(g->tuned & GG_TUNE_PR) && recall(k, p)) g->pr_shape = gg_pull_shape{p.v[0], p.v[1], p.v[2]};
    k.family = GG_TUNE_SPMV;
    if (!(g->tuned & GG_TUNE_SPMV) && recall(k, p)) g->spmv_shape = gg_pull_shape{p.v[0], p.v[1], p.v[2]};
    k.family = GG_TUNE_BFS;
    if (!(g->tuned & GG_TUNE_BFS) && recall(k, p)) g->bfs_heavy = p.v[0];
    k.family = GG_TUNE_PPR;
    if (!(g->tuned & GG_TUNE_PPR) && recall(k, p)) g->ppr_tile = p.v[0];
}

extern "C" gg_status gg_autotune(gg_graph *g, const gg_tune_params *p, gg_tune_result *r, void *stream)
{
    GgRange range("gg_autotune");
    if (!g || !p) return gg_fail(GG_ERR_INVALID, "NULL argument");
    if (p->storage > 2) return gg_fail(GG_ERR_INVALID, "unknown storage");
    if ((p->families & GG_TUNE_BATCH) && (!p->vertex_off || !p->ngraphs))
        return gg_fail(GG_ERR_INVALID, "GG_TUNE_BATCH needs the batch's vertex_off");
    cudaStream_t s = gg_stream(g, stream);
    g->tune_looked_up = true; /* the picks made here win over remembered ones */
    const uint32_t reps = p->reps ? p->reps : 3;
    gg_tune_result res;
    memset(&res, 0, sizeof(res));
    Key k{};
    GG_CHECK(graph_class(g, s, k));
    auto note = [&](const gg_tune_choice &c, uint32_t storage) {
        res.choice[res.n++] = c;
        Key kk = k;
        kk.family = c.family;
        kk.storage = storage;
        if (c.family == GG_TUNE_BATCH) kk.glog = ilog2((double)p->ngraphs);
        remember(kk, Pick{{c.params[0], c.params[1], c.params[2], c.params[3], c.params[4]}});
        g->tuned |= c.family;
    };
    if ((p->families & GG_TUNE_PR) && g->in_off)
    {
        gg_tune_choice c{};
        GG_CHECK(tune_pull(g, false, p->storage, reps, s, c));
        note(c, 0);
    }
    if ((p->families & GG_TUNE_SPMV) && g->in_off && g->in_w)
    {
        gg_tune_choice c{};
        GG_CHECK(tune_pull(g, true, p->storage, reps, s, c));
        note(c, 0);
    }
    if ((p->families & GG_TUNE_BFS) && g->out_off && g->in_off)
    {
        gg_tune_choice c{};
        GG_CHECK(tune_bfs(g, reps, s, c));
        if (c.family) note(c, 0);
    }
    if ((p->families & GG_TUNE_PPR) && g->in_off)
    {
        gg_tune_choice c{};
        GG_CHECK(tune_ppr(g, p->storage, reps, s, c));
        if (c.family) note(c, 0);
    }
    if ((p->families & GG_TUNE_BATCH) && g->in_off)
    {
        gg_tune_choice c{};
        GG_CHECK(tune_batch(g, p->ngraphs, p->vertex_off, reps, s, c));
        note(c, 0);
    }
    if (r) *r = res;
    return GG_OK;
}

extern "C" gg_status gg_tune_save(const char *path)
{
    if (!path) return gg_fail(GG_ERR_INVALID, "NULL path");
    FILE *f = fopen(path, "w");
    if (!f) return gg_fail(GG_ERR_INVALID, std::string("cannot write ") + path);
    std::lock_guard<std::mutex> lk(g_mu);
    fprintf(f, "# family storage log2V log2deg log2skew sms log2graphs : p0 p1 p2 p3 p4\n");
    for (const auto &e : g_cache)
        fprintf(f, "%u %u %u %u %u %u %u : %u %u %u %u %u\n", e.first.family, e.first.storage, e.first.vlog,
                e.first.dlog, e.first.slog, e.first.sms, e.first.glog, e.second.v[0], e.second.v[1], e.second.v[2],
                e.second.v[3], e.second.v[4]);
    const bool ok = fclose(f) == 0;
    return ok ? GG_OK : gg_fail(GG_ERR_INVALID, std::string("cannot write ") + path);
}

extern "C" gg_status gg_tune_load(const char *path)
{
    if (!path) return gg_fail(GG_ERR_INVALID, "NULL path");
    FILE *f = fopen(path, "r");
    if (!f) return gg_fail(GG_ERR_INVALID, std::string("cannot read ") + path);
    char line[256];
    uint32_t n = 0;
    while (fgets(line, sizeof line, f))
    {
        Key k{};
        Pick p{};
        if (line[0] == '#') continue;
        if (sscanf(line, "%u %u %u %u %u %u %u : %u %u %u %u %u", &k.family, &k.storage, &k.vlog, &k.dlog, &k.slog,
                   &k.sms, &k.glog, &p.v[0], &p.v[1], &p.v[2], &p.v[3], &p.v[4]) == 12)
        {
            remember(k, p);
            n++;
        }
    }
    fclose(f);
    return GG_OK;
}

extern "C" gg_status gg_tune_reset(void)
{
    std::lock_guard<std::mutex> lk(g_mu);
    g_cache.clear();
    return GG_OK;
}

extern "C" gg_status gg_tune_get(const gg_graph *g, uint32_t family, uint32_t *params)
{
    if (!g || !params) return gg_fail(GG_ERR_INVALID, "NULL argument");
    memset(params, 0, 5 * sizeof(uint32_t));
    switch (family)
    {
    case GG_TUNE_PR: params[0] = g->pr_shape.hot; params[1] = g->pr_shape.ctas; params[2] = g->pr_shape.hot_warps; break;
    case GG_TUNE_SPMV:
        params[0] = g->spmv_shape.hot; params[1] = g->spmv_shape.ctas; params[2] = g->spmv_shape.hot_warps; break;
    case GG_TUNE_BFS: params[0] = g->bfs_heavy; break;
    case GG_TUNE_PPR: params[0] = g->ppr_tile; break;
    case GG_TUNE_BATCH:
        params[0] = g->graphs_cfg.ipt; params[1] = g->graphs_cfg.warps; params[2] = g->graphs_cfg.smem_vmax;
        params[3] = g->graphs_cfg.ctas; params[4] = g->graphs_cfg.strategy; break;
    default: return gg_fail(GG_ERR_INVALID, "unknown tuning family");
    }
    return GG_OK;
}
