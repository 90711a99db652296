/*
 * PageRank of many independent graphs in one persistent launch.
 *
 * The mapping holds the block-diagonal union of `ngraphs` graphs (graph i:
 * rows vertex_off[i] .. vertex_off[i+1], its in-edges contiguous in the
 * CSC).  Per graph the arithmetic is the reference's pull PageRank
 * (02_capi_graph/src/algorithms/capi/pageRank.c:1026-1085: contribution =
 * rank / outdeg, rank' = 0.15 + 0.85 * sum, stop when no vertex moved by
 * epsilon, divide by the graph's V at the end), each graph with its own
 * stop.
 *
 * One CTA ranks one graph at a time, all of its iterations, with only CTA
 * barriers between the gather and the vertex pass; CTAs take graphs from a
 * counter, largest first, so the longest graphs start early and the small
 * ones fill in.  The gather is the merge-path warp engine over tiles cut
 * per graph.  Two bins: a graph of at most `smem_vmax` vertices keeps its
 * contributions and row sums in shared memory (the gather reads shared
 * memory, not L2); a larger one keeps them in global memory (L2).  Tile
 * size (IPT), warps per CTA and the bin threshold are chosen by the
 * autotuner (tune.cu) or set by the caller.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "gg_device.cuh"

namespace {

using namespace gg;

__device__ __forceinline__ float contrib_of_f(float rank, uint32_t deg)
{
    return deg ? __fdiv_rn(rank, __uint2float_rn(deg)) : 0.0f;
}

struct GraphsArgs
{
    const uint32_t *off, *adj, *outdeg;
    const uint32_t *voff;   /* ngraphs + 1 */
    const uint32_t *order;  /* graph ids, largest first */
    const uint32_t *cbase;  /* ngraphs + 1: graph g's tile coordinates are coord[cbase[g] .. cbase[g+1]) */
    const uint2 *coord;
    float *rank, *contrib, *sums; /* union-sized; contrib and sums used by graphs above smem_vmax */
    uint32_t *counter;      /* next graph to take */
    uint32_t *iters_out;    /* per graph: the reference's iteration count */
    uint32_t *active_out;   /* per graph: active vertices of its last iteration */
    double *err_out;        /* per graph: last iteration's sum |delta| / V */
    uint32_t ngraphs, V, iterations, smem_vmax, one_over_n;
    float damp, eps_f;
};

/* the in-neighbour's contribution: shared memory for small graphs, global
 * (plain loads: the values are rewritten inside the launch, by the same
 * CTA) otherwise; `base` is offset by the graph's first vertex so it takes
 * union ids.  One engine instance serves both through a generic pointer: a
 * second instance for the global case made the kernel spill at its 64
 * registers. */
struct GraphsGather
{
    typedef float Acc;
    typedef float Raw;
    const float *base;
    __device__ __forceinline__ Raw load(uint32_t, uint32_t u) const { return base[u]; }
    __device__ __forceinline__ Acc value(const Raw &r) const { return r; }
};

/* every iteration of one graph (vertices vb .. vb + Vg) by the whole CTA:
 * the gather into sm, a CTA barrier, the vertex pass (two vertices per
 * thread per step... 's residual and
 * active count; returns the reference's iteration count */
template <int IPT>
__device__ __forceinline__ uint32_t graph_iterations(const GraphsArgs &a, unsigned char *stage, float *c, float *sm,
                                                     uint32_t vb, uint32_t Vg, uint32_t cb, uint32_t ntiles,
                                                     float base, double *err_out, uint32_t *act_out)
{
    typedef PullStage<IPT, float> S;
    __shared__ double s_err[32];
    __shared__ uint32_t s_act[32];
    const uint32_t warps = blockDim.x >> 5, w = threadIdx.x >> 5;
    uint32_t it = 0, act = 0;
    double err = 0.0;
    for (; it < a.iterations; it++)
    {
        warp_pull_sums_core<IPT>(reinterpret_cast<uint32_t *>(stage), reinterpret_cast<float *>(stage + S::OFF_BYTES),
                                 reinterpret_cast<float *>(stage + S::OFF_BYTES + S::VAL_BYTES), w, warps, a.off,
                                 a.adj, a.V, a.coord + cb, ntiles, sm - vb, GraphsGather{c - vb});
        __syncthreads();
        double e_sum = 0.0;
        uint32_t n_act = 0;
        constexpr uint32_t U = 2; /* measured: 4 was slower, and spills at IPT 9 */
        for (uint32_t v0 = threadIdx.x; v0 < Vg; v0 += U * blockDim.x)
        {
            float sv[U], pr[U];
            uint32_t dg[U];
#pragma unroll
            for (uint32_t k = 0; k < U; k++)
            {
                const uint32_t v = v0 + k * blockDim.x;
                if (v < Vg)
                {
                    sv[k] = sm[v];
                    pr[k] = a.rank[vb + v];
                    dg[k] = __ldg(a.outdeg + vb + v);
                }
            }
#pragma unroll
            for (uint32_t k = 0; k < U; k++)
            {
                const uint32_t v = v0 + k * blockDim.x;
                if (v < Vg)
                {
                    sm[v] = 0.0f;
                    const float nr = __fadd_rn(base, __fmul_rn(a.damp, sv[k]));
                    a.rank[vb + v] = nr;
                    const float e = fabsf(__fsub_rn(nr, pr[k]));
                    e_sum += (double)e;
                    n_act += e >= a.eps_f ? 1u : 0u;
                    c[v] = contrib_of_f(nr, dg[k]);
                }
            }
        }
        /* CTA sums of the residual and the active count */
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
        {
            e_sum += __shfl_down_sync(0xffffffffu, e_sum, o);
            n_act += __shfl_down_sync(0xffffffffu, n_act, o);
        }
        if ((threadIdx.x & 31) == 0)
        {
            s_err[w] = e_sum;
            s_act[w] = n_act;
        }
        __syncthreads();
        err = 0.0;
        act = 0;
        for (uint32_t k = 0; k < warps; k++)
        {
            err += s_err[k];
            act += s_act[k];
        }
        __syncthreads();
        if (act == 0) break; /* pageRank.c:1073: the reference stops here */
    }
    *err_out = err;
    *act_out = act;
    return it < a.iterations ? it : a.iterations;
}

template <int IPT>
__global__ void __launch_bounds__(1024, 1) k_pr_graphs(GraphsArgs a)
{
    extern __shared__ __align__(16) unsigned char gg_dyn[];
    typedef PullStage<IPT, float> S;
    const uint32_t warps = blockDim.x >> 5, w = threadIdx.x >> 5;
    unsigned char *stage = gg_dyn + (size_t)w * S::BYTES;
    float *s_c = reinterpret_cast<float *>(gg_dyn + (size_t)warps * S::BYTES);
    float *s_sum = s_c + a.smem_vmax;
    __shared__ uint32_t s_g;
    for (;;)
    {
        if (threadIdx.x == 0) s_g = atomicAdd(a.counter, 1u);
        __syncthreads();
        const uint32_t gidx = s_g;
        __syncthreads();
        if (gidx >= a.ngraphs) return;
        const uint32_t gi = a.order[gidx];
        const uint32_t vb = a.voff[gi], Vg = a.voff[gi + 1] - vb;
        const uint32_t cb = a.cbase[gi], ntiles = a.cbase[gi + 1] - cb - 1;
        const bool small = Vg <= a.smem_vmax;
        float *c = small ? s_c : a.contrib + vb;
        float *sm = small ? s_sum : a.sums + vb;
        const float base_pr = __fsub_rn(1.0f, a.damp);
        const float fV = __uint2float_rn(Vg ? Vg : 1u);
        const float base = a.one_over_n ? __fdiv_rn(base_pr, fV) : base_pr;
        const float init = a.one_over_n ? __fdiv_rn(1.0f, fV) : base_pr;
        for (uint32_t v = threadIdx.x; v < Vg; v += blockDim.x)
        {
            a.rank[vb + v] = init;
            c[v] = contrib_of_f(init, a.outdeg[vb + v]);
            sm[v] = 0.0f;
        }
        __syncthreads();
        double err = 0.0;
        uint32_t act = 0, its;
        its = graph_iterations<IPT>(a, stage, c, sm, vb, Vg, cb, ntiles, base, &err, &act);
        /* pageRank.c:1080-1085 */
        if (!a.one_over_n)
            for (uint32_t v = threadIdx.x; v < Vg; v += blockDim.x)
                a.rank[vb + v] = __fdiv_rn(a.rank[vb + v], fV);
        if (threadIdx.x == 0)
        {
            a.iters_out[gi] = its;
            a.active_out[gi] = act;
            a.err_out[gi] = Vg ? err / (double)Vg : 0.0;
        }
        __syncthreads();
    }
}

/* tile coordinates of every graph's own merge path, in union indices:
 * graph g has ntiles_g = ceil((V_g + E_g) / items) tiles and ntiles_g + 1
 * coordinates from cbase[g] */
__global__ void k_graph_tile_coords(const uint32_t *__restrict__ off, const uint32_t *__restrict__ voff,
                                    const uint32_t *__restrict__ cbase, uint32_t ngraphs, uint32_t items,
                                    uint2 *__restrict__ coord)
{
    const uint32_t total = cbase[ngraphs];
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x)
    {
        uint32_t lo = 0, hi = ngraphs - 1;
        while (lo < hi)
        {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (cbase[mid] <= t)
                lo = mid;
            else
                hi = mid - 1;
        }
        const uint32_t g = lo, vb = voff[g], Vg = voff[g + 1] - vb;
        const uint32_t eb = off[vb], Eg = off[vb + Vg] - eb;
        const uint64_t n = (uint64_t)Vg + Eg;
        uint64_t d = (uint64_t)(t - cbase[g]) * items;
        if (d > n) d = n;
        /* rows of the graph ended before diagonal d */
        uint64_t r0 = d > Eg ? d - Eg : 0, r1 = d < Vg ? d : Vg;
        while (r0 < r1)
        {
            const uint64_t mid = (r0 + r1) >> 1;
            if ((uint64_t)(off[vb + mid + 1] - eb) + mid < d)
                r0 = mid + 1;
            else
                r1 = mid;
        }
        coord[t] = make_uint2(vb + (uint32_t)r0, eb + (uint32_t)(d - r0));
    }
}

/* every in-neighbour of a row lies in the row's own graph (the kernel reads
 * a small graph's contributions from shared memory by local index); sets
 * *bad otherwise */
__global__ void k_check_block_diagonal(const uint32_t *__restrict__ off, const uint32_t *__restrict__ adj,
                                       const uint32_t *__restrict__ voff, uint32_t ngraphs, uint32_t *bad)
{
    const uint32_t V = voff[ngraphs];
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
    {
        uint32_t lo = 0, hi = ngraphs - 1;
        while (lo < hi)
        {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (voff[mid] <= v)
                lo = mid;
            else
                hi = mid - 1;
        }
        const uint32_t a = voff[lo], b = voff[lo + 1];
        for (uint32_t j = off[v]; j < off[v + 1]; j++)
        {
            const uint32_t u = adj[j];
            if (u < a || u >= b)
            {
                atomicExch(bad, 1u);
                break;
            }
        }
    }
}

__global__ void k_gather_offsets(const uint32_t *__restrict__ off, const uint32_t *__restrict__ idx, uint32_t n,
                                 uint32_t *__restrict__ out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = off[idx[i]];
}

template <int IPT>
size_t graphs_smem(uint32_t warps, uint32_t smem_vmax)
{
    return (size_t)warps * PullStage<IPT, float>::BYTES + (size_t)smem_vmax * 8;
}

} // namespace

/* per-call state of the many-graphs run, cached on the mapping: the graph
 * boundaries it was cut for, the tile coordinates and the size order */
gg_status gg_graphs_prepare(gg_graph *g, uint32_t ngraphs, const uint32_t *h_voff, uint32_t items, cudaStream_t s)
{
    gg_graphs_state &st = g->graphs;
    if (st.ngraphs == ngraphs && st.items == items && st.h_voff.size() == (size_t)ngraphs + 1 &&
        std::equal(st.h_voff.begin(), st.h_voff.end(), h_voff))
        return GG_OK;
    for (uint32_t i = 0; i < ngraphs; i++)
        if (h_voff[i + 1] < h_voff[i] || h_voff[i + 1] > g->V)
            return gg_fail(GG_ERR_INVALID, "vertex_off must be non-decreasing and end at most at V");
    /* each graph's edge count: the CSC offsets at the boundaries */
    std::vector<uint32_t> h_off(ngraphs + 1);
    void *d_tmp;
    GG_CHECK(gg_work(g, 31, ((size_t)ngraphs + 1) * 8 + 16, &d_tmp));
    uint32_t *d_v = (uint32_t *)d_tmp, *d_o = d_v + ngraphs + 1;
    GG_CUDA(cudaMemcpyAsync(d_v, h_voff, ((size_t)ngraphs + 1) * 4, cudaMemcpyHostToDevice, s));
    k_gather_offsets<<<(ngraphs + 256) / 256, 256, 0, s>>>(g->in_off, d_v, ngraphs + 1, d_o);
    GG_CUDA(cudaGetLastError());
    uint32_t *d_bad = d_o + ngraphs + 1, *h_bad = nullptr;
    GG_CHECK(gg_pinned(g, 64, (void **)&h_bad));
    GG_CUDA(cudaMemsetAsync(d_bad, 0, 4, s));
    if (h_voff[ngraphs] > h_voff[0])
        k_check_block_diagonal<<<gg_sm_count() * 8, 256, 0, s>>>(g->in_off, g->in_adj, d_v, ngraphs, d_bad);
    GG_CUDA(cudaGetLastError());
    GG_CHECK(gg_wait(s)); /* bounded, before a copy to pageable memory */
    GG_CUDA(cudaMemcpyAsync(h_off.data(), d_o, ((size_t)ngraphs + 1) * 4, cudaMemcpyDeviceToHost, s));
    GG_CUDA(cudaMemcpyAsync(h_bad, d_bad, 4, cudaMemcpyDeviceToHost, s));
    GG_CHECK(gg_wait(s));
    if (*h_bad) return gg_fail(GG_ERR_INVALID, "edges cross the graph boundaries of vertex_off");
    std::vector<uint32_t> cbase(ngraphs + 1), order(ngraphs);
    uint64_t acc = 0;
    for (uint32_t i = 0; i < ngraphs; i++)
    {
        cbase[i] = (uint32_t)acc;
        const uint64_t n = (uint64_t)(h_voff[i + 1] - h_voff[i]) + (h_off[i + 1] - h_off[i]);
        acc += (n + items - 1) / items + 1;
        if (acc >= 0xffffffffull) return gg_fail(GG_ERR_INVALID, "too many tiles");
    }
    cbase[ngraphs] = (uint32_t)acc;
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) {
        return (uint64_t)(h_voff[x + 1] - h_voff[x]) + (h_off[x + 1] - h_off[x]) >
               (uint64_t)(h_voff[y + 1] - h_voff[y]) + (h_off[y + 1] - h_off[y]);
    });
    if (st.coord) gg_dev_free(g, st.coord, st.bytes);
    st.coord = nullptr;
    st.ngraphs = 0;
    /* one allocation: voff, cbase, order, then the coordinates (8-byte aligned) */
    const size_t words = (size_t)(ngraphs + 1) * 2 + ngraphs;
    const size_t head = (words * 4 + 15) / 16 * 16;
    st.bytes = head + (size_t)acc * sizeof(uint2);
    GG_CHECK(gg_dev_alloc(g, &st.coord, st.bytes));
    uint32_t *d = (uint32_t *)st.coord;
    std::vector<uint32_t> packed;
    packed.reserve(words);
    packed.insert(packed.end(), h_voff, h_voff + ngraphs + 1);
    packed.insert(packed.end(), cbase.begin(), cbase.end());
    packed.insert(packed.end(), order.begin(), order.end());
    GG_CUDA(cudaMemcpyAsync(d, packed.data(), words * 4, cudaMemcpyHostToDevice, s));
    st.voff = d;
    st.cbase = d + ngraphs + 1;
    st.order = d + 2 * ((size_t)ngraphs + 1);
    st.tiles = (uint2 *)((char *)st.coord + head);
    k_graph_tile_coords<<<gg_sm_count() * 8, 256, 0, s>>>(g->in_off, st.voff, st.cbase, ngraphs, items, st.tiles);
    GG_CUDA(cudaGetLastError());
    GG_CHECK(gg_wait(s));
    st.h_voff.assign(h_voff, h_voff + ngraphs + 1);
    st.ngraphs = ngraphs;
    st.items = items;
    return GG_OK;
}

/* one launch: every graph, every iteration; per-graph results into the
 * device arrays iters/active/err (ngraphs each) */
gg_status gg_graphs_launch(gg_graph *g, const gg_graphs_config &cfg, uint32_t ngraphs, const gg_pr_params *p,
                           float eps_f, float *rank, uint32_t *counter, uint32_t *iters, uint32_t *active, double *err,
                           cudaStream_t s)
{
    const gg_graphs_state &st = g->graphs;
    void *c, *sums;
    GG_CHECK(gg_work(g, 2, ((size_t)g->V + 16) * 4, &c));
    GG_CHECK(gg_work(g, 5, ((size_t)g->V + 16) * 4, &sums));
    GraphsArgs a;
    a.off = g->in_off; a.adj = g->in_adj; a.outdeg = g->out_deg;
    a.voff = st.voff; a.order = st.order; a.cbase = st.cbase; a.coord = st.tiles;
    a.rank = rank; a.contrib = (float *)c; a.sums = (float *)sums;
    a.counter = counter; a.iters_out = iters; a.active_out = active; a.err_out = err;
    a.ngraphs = ngraphs; a.V = g->V; a.iterations = p->max_iterations; a.smem_vmax = cfg.smem_vmax;
    a.one_over_n = p->init_one_over_n; a.damp = p->damp; a.eps_f = eps_f;
    GG_CUDA(cudaMemsetAsync(counter, 0, 4, s));
    const uint32_t warps = cfg.warps;
    const void *fn = nullptr;
    size_t smem = 0;
    switch (cfg.ipt)
    {
    case 5: fn = (const void *)k_pr_graphs<5>; smem = graphs_smem<5>(warps, cfg.smem_vmax); break;
    case 9: fn = (const void *)k_pr_graphs<9>; smem = graphs_smem<9>(warps, cfg.smem_vmax); break;
    default: fn = (const void *)k_pr_graphs<7>; smem = graphs_smem<7>(warps, cfg.smem_vmax); break;
    }
    if (smem + 1024 > 227 * 1024) return gg_fail(GG_ERR_INVALID, "many-graphs configuration exceeds shared memory");
    GG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    /* carve-out: just the shared memory of cfg.ctas CTAs (1 KB reserved
     * each, plus the static part), so the rest of the SM's array stays L1
     * for the gathers' lines in flight */
    int dev = 0, smem_sm = 0;
    GG_CUDA(cudaGetDevice(&dev));
    GG_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
    cudaFuncAttributes fa;
    GG_CUDA(cudaFuncGetAttributes(&fa, fn));
    const uint32_t want = cfg.ctas ? cfg.ctas : 1;
    if (smem_sm > 0)
    {
        const double need = (double)want * (double)(smem + fa.sharedSizeBytes + 1024);
        int pct = (int)ceil(100.0 * need / (double)smem_sm);
        pct = pct < 1 ? 1 : (pct > 100 ? 100 : pct);
        GG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, pct));
    }
    int per_sm = 0;
    GG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, (int)(warps * 32), smem));
    if (per_sm < 1) return gg_fail(GG_ERR_INVALID, "many-graphs configuration cannot be resident");
    if ((uint32_t)per_sm > want) per_sm = (int)want;
    const uint32_t grid = std::min<uint32_t>((uint32_t)gg_sm_count() * (uint32_t)per_sm, ngraphs);
    void *args[] = {&a};
    GG_CUDA(cudaLaunchKernel(fn, dim3(grid ? grid : 1), dim3(warps * 32), args, smem, s));
    return GG_OK;
}

size_t gg_graphs_tile_items(const gg_graphs_config &cfg) { return (size_t)32 * (cfg.ipt == 5 || cfg.ipt == 9 ? cfg.ipt : 7); }


extern "C" gg_status gg_pagerank_batch_iterations(const gg_graph *g, uint32_t ngraphs, uint32_t *iterations)
{
    if (!g || !iterations) return gg_fail(GG_ERR_INVALID, "NULL argument");
    if (!g->graphs_iters || ngraphs != g->graphs_n)
        return gg_fail(GG_ERR_INVALID, "no many-graphs run with that many graphs on this mapping");
    GG_CUDA(cudaMemcpy(iterations, g->graphs_iters, (size_t)ngraphs * 4, cudaMemcpyDeviceToHost)); /* after the run's own bounded wait */
    return GG_OK;
}

extern "C" gg_status gg_pagerank_batch_config(gg_graph *g, uint32_t ipt, uint32_t warps, uint32_t smem_vmax,
                                              uint32_t ctas_per_sm)
{
    if (!g) return gg_fail(GG_ERR_INVALID, "NULL graph");
    if (ipt != 5 && ipt != 7 && ipt != 9) return gg_fail(GG_ERR_INVALID, "ipt must be 5, 7 or 9");
    if (warps < 1 || warps > 32) return gg_fail(GG_ERR_INVALID, "warps must be 1..32");
    if (ctas_per_sm < 1 || ctas_per_sm * warps > 64) return gg_fail(GG_ERR_INVALID, "ctas_per_sm must be 1..64/warps");
    gg_graphs_config c;
    c.ipt = ipt;
    c.warps = warps;
    c.smem_vmax = smem_vmax;
    c.ctas = ctas_per_sm;
    size_t smem = 0;
    switch (ipt)
    {
    case 5: smem = graphs_smem<5>(warps, smem_vmax); break;
    case 9: smem = graphs_smem<9>(warps, smem_vmax); break;
    default: smem = graphs_smem<7>(warps, smem_vmax); break;
    }
    if (smem + 1024 > 227 * 1024 || ctas_per_sm * (smem + 2048) > 228 * 1024)
        return gg_fail(GG_ERR_INVALID, "configuration exceeds shared memory");
    c.strategy = g->graphs_cfg.strategy;
    g->graphs_cfg = c;
    g->tuned |= GG_TUNE_BATCH;
    return GG_OK;
}

extern "C" gg_status gg_pagerank_batch_strategy(gg_graph *g, uint32_t strategy)
{
    if (!g) return gg_fail(GG_ERR_INVALID, "NULL graph");
    if (strategy > 2) return gg_fail(GG_ERR_INVALID, "strategy must be 0, 1 or 2");
    g->graphs_cfg.strategy = strategy;
    g->tuned |= GG_TUNE_BATCH;
    return GG_OK;
}
