/*
 * Connected components on CSR (connectedComponents.c:337-720) on one GPU.
 *
 * Every algorithm ends with each vertex labelled by the smallest vertex id
 * of its weakly connected component; the labels are deterministic, the
 * iteration counts (as in the reference) depend on the order of concurrent
 * updates.  Edge passes walk the CSR in merge-path tiles (warp_push), so a
 * hub's edges are spread over many warps.
 *
 *   Shiloach-Vishkin (pushpull 0; :362-468 with the FPGA hook step of
 *     cu_ConnectedComponents/.../cu_update_kernel_control.sv:171-190):
 *     repeat { k_cc_hook: for every out-edge, the higher of the two labels,
 *     if it is still a root, is pointed at the lower one; k_cc_compress:
 *     pointer jumping to the root } while any hook happened
 *   Afforest (pushpull 1 and default; :470-626): `neighbor_rounds` rounds of
 *     k_cc_link_round (link u with its r-th out-neighbour) + compression; a
 *     sample of labels picks the largest component, whose vertices skip the
 *     final link (k_cc_link_rest over the remaining out-edges and, when the
 *     CSC is mapped, every in-edge); compression
 *   weakly connected components (pushpull 2; :628-720): repeat k_cc_minprop
 *     (both endpoints of every out-edge take the smaller label by atomicMin)
 *     while any label fell
 *
 * cc_link is the reference's linkNodes (:249-269): union by the lower label
 * with a compare-and-swap on the higher root, retried while the roots move.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "gg_device.cuh"

namespace {

using namespace gg;

struct CcFlags
{
    unsigned int changed;
    unsigned int err;
    unsigned int roots;
    unsigned int pad;
};

constexpr uint32_t LINK_RETRIES = 1u << 16;

__device__ __forceinline__ uint32_t ld_comp(const uint32_t *comp, uint32_t i)
{
    return *(const volatile uint32_t *)(comp + i);
}

__device__ __forceinline__ void cc_link(uint32_t u, uint32_t v, uint32_t *comp, CcFlags *f)
{
    uint32_t a = ld_comp(comp, u), b = ld_comp(comp, v);
    for (uint32_t tries = 0; a != b; tries++)
    {
        if (tries == LINK_RETRIES)
        {
            atomicOr(&f->err, 1u);
            return;
        }
        const uint32_t hi = a > b ? a : b, lo = a > b ? b : a;
        const uint32_t ph = ld_comp(comp, hi);
        if (ph == lo) return;
        if (ph == hi && atomicCAS(comp + hi, hi, lo) == hi) return;
        a = ld_comp(comp, ld_comp(comp, hi));
        b = ld_comp(comp, lo);
    }
}

__global__ void k_cc_init(uint32_t *comp, uint32_t V)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) comp[v] = v;
}

/* pointer jumping until every vertex points at its root (labels only
 * decrease along a chain, so each loop ends) */
__global__ void k_cc_compress(uint32_t *comp, uint32_t V)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
    {
        uint32_t c = ld_comp(comp, v);
        uint32_t cc = ld_comp(comp, c);
        while (c != cc)
        {
            c = cc;
            cc = ld_comp(comp, c);
        }
        comp[v] = c;
    }
}

__global__ void __launch_bounds__(GG_TILE_NT) k_cc_hook(const uint32_t *__restrict__ off,
                                                        const uint32_t *__restrict__ adj, const uint2 *__restrict__ coord,
                                                        uint32_t ntiles, uint32_t V, uint32_t *comp, CcFlags *f)
{
    /* the row's label is read once per row segment; a label read here may
     * be older than another warp's hook in the same pass, which costs at most
     * a repeat in the next pass (a pass that hooks nothing reads no stale
     * value, so the stop test is exact) */
    struct Op
    {
        typedef uint32_t RowVal;
        uint32_t *comp;
        CcFlags *f;
        __device__ __forceinline__ uint32_t row_value(uint32_t r) const { return comp[r]; }
        __device__ __forceinline__ void scatter(uint32_t cu, uint32_t, uint32_t v) const
        {
            const uint32_t cv = comp[v];
            if (cu == cv) return;
            const uint32_t hi = cu > cv ? cu : cv, lo = cu > cv ? cv : cu;
            if (comp[hi] == hi)
            {
                comp[hi] = lo;
                *(volatile unsigned int *)&f->changed = 1u;
            }
        }
    } op{comp, f};
    warp_push<GG_TILE_IPT, GG_TILE_WARPS>(off, adj, V, coord, ntiles, op);
}

__global__ void __launch_bounds__(GG_TILE_NT) k_cc_minprop(const uint32_t *__restrict__ off,
                                                           const uint32_t *__restrict__ adj,
                                                           const uint2 *__restrict__ coord, uint32_t ntiles,
                                                           uint32_t V, uint32_t *comp, CcFlags *f)
{
    /* the row's label is read once per row segment (a stale, larger label
     * only propagates less in this pass) */
    struct Row
    {
        uint32_t u, cu;
    };
    struct Op
    {
        typedef Row RowVal;
        uint32_t *comp;
        CcFlags *f;
        __device__ __forceinline__ Row row_value(uint32_t r) const { return Row{r, comp[r]}; }
        __device__ __forceinline__ void scatter(const Row &rv, uint32_t, uint32_t v) const
        {
            const uint32_t cv = comp[v];
            if (rv.cu < cv)
            {
                if (atomicMin(comp + v, rv.cu) > rv.cu) *(volatile unsigned int *)&f->changed = 1u;
            }
            else if (cv < rv.cu)
            {
                if (atomicMin(comp + rv.u, cv) > cv) *(volatile unsigned int *)&f->changed = 1u;
            }
        }
    } op{comp, f};
    warp_push<GG_TILE_IPT, GG_TILE_WARPS>(off, adj, V, coord, ntiles, op);
}

__global__ void k_cc_link_round(const uint32_t *__restrict__ off, const uint32_t *__restrict__ adj, uint32_t V,
                                uint32_t r, uint32_t *comp, CcFlags *f)
{
    for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < V; u += gridDim.x * blockDim.x)
    {
        const uint32_t j = off[u] + r;
        if (j < off[u + 1]) cc_link(u, adj[j], comp, f);
    }
}

/* the final link: every edge of a row whose label is not `skip`, from the
 * row's `first` + `skip_head` edge on (out-edges skip the rounds already
 * linked, in-edges none) */
__global__ void __launch_bounds__(GG_TILE_NT) k_cc_link_rest(const uint32_t *__restrict__ off,
                                                             const uint32_t *__restrict__ adj,
                                                             const uint2 *__restrict__ coord, uint32_t ntiles,
                                                             uint32_t V, uint32_t skip_head, uint32_t skip,
                                                             uint32_t *comp, CcFlags *f)
{
    struct Row
    {
        uint32_t u, first;
        bool skip;
    };
    struct Op
    {
        typedef Row RowVal;
        const uint32_t *off;
        uint32_t skip_head, skip;
        uint32_t *comp;
        CcFlags *f;
        __device__ __forceinline__ Row row_value(uint32_t r) const
        {
            return Row{r, off[r] + skip_head, ld_comp(comp, r) == skip};
        }
        __device__ __forceinline__ void scatter(const Row &rv, uint32_t j, uint32_t v) const
        {
            if (!rv.skip && j >= rv.first) cc_link(rv.u, v, comp, f);
        }
    } op{off, skip_head, skip, comp, f};
    warp_push<GG_TILE_IPT, GG_TILE_WARPS>(off, adj, V, coord, ntiles, op);
}

__global__ void k_cc_sample(const uint32_t *__restrict__ comp, uint32_t V, uint64_t seed, uint32_t n, uint32_t *out)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        /* SplitMix64 of seed + i */
        uint64_t z = seed + i;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        out[i] = comp[z % V];
    }
}

__global__ void k_cc_roots(const uint32_t *__restrict__ comp, uint32_t V, CcFlags *f)
{
    uint32_t n = 0;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) n += comp[v] == v;
    n = warp_sum(n);
    if ((threadIdx.x & 31) == 0 && n) atomicAdd(&f->roots, n);
}

int grid_for(uint32_t n)
{
    const uint32_t b = (n + 255) / 256, cap = (uint32_t)gg_sm_count() * 8;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

struct Cc
{
    gg_graph *g;
    cudaStream_t s;
    uint32_t *comp;
    CcFlags *f, *h;
    uint32_t launches = 0;
    int profile = 0;
    std::vector<cudaEvent_t> evs;
};

gg_status mark(Cc &C)
{
    if (!C.profile) return GG_OK;
    cudaEvent_t e;
    GG_CHECK(gg_event_at(C.g, (uint32_t)C.evs.size(), &e));
    GG_CUDA(cudaEventRecord(e, C.s));
    C.evs.push_back(e);
    return GG_OK;
}

gg_status read_flags(Cc &C)
{
    GG_CUDA(cudaMemcpyAsync(C.h, C.f, sizeof(CcFlags), cudaMemcpyDeviceToHost, C.s));
    GG_CHECK(gg_wait(C.s));
    if (C.h->err) return gg_fail(GG_ERR_KERNEL, "connected components: a link gave up after its retry limit");
    return GG_OK;
}

gg_status compress(Cc &C)
{
    k_cc_compress<<<grid_for(C.g->V), 256, 0, C.s>>>(C.comp, C.g->V);
    C.launches++;
    GG_CUDA(cudaGetLastError());
    return GG_OK;
}

/* repeat one edge pass + (for SV) compression while a label changed */
template <class Launch>
gg_status until_stable(Cc &C, uint32_t max_iterations, bool with_compress, uint32_t *iterations, Launch launch)
{
    uint32_t it = 0;
    for (;;)
    {
        GG_CUDA(cudaMemsetAsync(&C.f->changed, 0, 4, C.s));
        GG_CHECK(mark(C));
        launch();
        C.launches++;
        if (with_compress) GG_CHECK(compress(C));
        GG_CHECK(mark(C));
        GG_CUDA(cudaGetLastError());
        it++;
        GG_CHECK(read_flags(C));
        if (!C.h->changed) break;
        if (it >= max_iterations) return gg_fail(GG_ERR_KERNEL, "connected components did not settle");
    }
    *iterations = it;
    return GG_OK;
}

} // namespace

extern "C" gg_status gg_cc(gg_graph *g, const gg_cc_params *p, uint32_t *components, gg_cc_result *r, void *stream)
{
    GgRange range("gg_cc");
    if (!g || !p) return gg_fail(GG_ERR_INVALID, "NULL argument");
    if (p->algorithm > 2) return gg_fail(GG_ERR_INVALID, "unknown connected-components algorithm");
    if (!g->out_off) return gg_fail(GG_ERR_INVALID, "connected components need GG_MAP_OUT");
    if (p->algorithm == GG_CC_AFFOREST && p->use_in_edges == 1 && !g->in_off)
        return gg_fail(GG_ERR_INVALID, "use_in_edges needs GG_MAP_IN");
    const uint32_t V = g->V;
    Cc C;
    C.g = g;
    C.s = gg_stream(g, stream);
    C.profile = (int)p->profile;
    void *ptr;
    GG_CHECK(gg_work(g, 0, ((size_t)V + 64) * 4, &ptr));
    C.comp = (uint32_t *)ptr;
    GG_CHECK(gg_work(g, 7, 256, &ptr));
    C.f = (CcFlags *)ptr;
    GG_CHECK(gg_pinned(g, 256, &ptr));
    C.h = (CcFlags *)ptr;
    GG_CUDA(cudaMemsetAsync(C.f, 0, sizeof(CcFlags), C.s));
    k_cc_init<<<grid_for(V), 256, 0, C.s>>>(C.comp, V);
    C.launches++;
    GG_CUDA(cudaGetLastError());

    gg_cc_result res{};
    const uint32_t max_it = p->max_iterations ? p->max_iterations : V + 1;
    gg_tiles *t = nullptr;
    GG_CHECK(gg_tiles_get(g, 0, C.s, &t));
    const int tgrid = gg_persistent_grid((const void *)k_cc_hook, t->ntiles);
    if (p->algorithm == 0)
    {
        GG_CHECK(until_stable(C, max_it, true, &res.iterations, [&] {
            k_cc_hook<<<tgrid, GG_TILE_NT, 0, C.s>>>(g->out_off, g->out_adj, t->coord, t->ntiles, V, C.comp, C.f);
        }));
    }
    else if (p->algorithm == 2)
    {
        GG_CHECK(until_stable(C, max_it, false, &res.iterations, [&] {
            k_cc_minprop<<<tgrid, GG_TILE_NT, 0, C.s>>>(g->out_off, g->out_adj, t->coord, t->ntiles, V, C.comp, C.f);
        }));
    }
    else
    {
        const uint32_t rounds = p->neighbor_rounds ? p->neighbor_rounds : 2;
        GG_CHECK(mark(C));
        for (uint32_t rr = 0; rr < rounds; rr++)
        {
            k_cc_link_round<<<grid_for(V), 256, 0, C.s>>>(g->out_off, g->out_adj, V, rr, C.comp, C.f);
            C.launches++;
            GG_CHECK(compress(C));
        }
        /* the skipped component: the most frequent label among the samples
         * (ties to the smaller label); none when in-edges are not linked and
         * the caller has not declared the graph symmetric */
        const bool use_in = p->use_in_edges == 1 || (p->use_in_edges == 2 && g->in_off);
        const bool may_skip = use_in || p->use_in_edges == 0;
        uint32_t skip = 0xffffffffu;
        const uint32_t ns = p->samples ? (p->samples < V ? p->samples : V) : (V < 1024 ? V : 1024);
        if (may_skip && ns)
        {
            void *sp;
            GG_CHECK(gg_work(g, 1, (size_t)ns * 4, &sp));
            k_cc_sample<<<grid_for(ns), 256, 0, C.s>>>(C.comp, V, p->seed, ns, (uint32_t *)sp);
            C.launches++;
            std::vector<uint32_t> smp(ns);
            GG_CHECK(gg_wait(C.s)); /* bounded, before a copy to pageable memory */
            GG_CUDA(cudaMemcpyAsync(smp.data(), sp, (size_t)ns * 4, cudaMemcpyDeviceToHost, C.s));
            GG_CHECK(gg_wait(C.s));
            std::sort(smp.begin(), smp.end());
            uint32_t best = 0;
            for (size_t i = 0; i < smp.size();)
            {
                size_t k = i;
                while (k < smp.size() && smp[k] == smp[i]) k++;
                if (k - i > best)
                {
                    best = (uint32_t)(k - i);
                    skip = smp[i];
                }
                i = k;
            }
        }
        res.skipped_label = skip;
        k_cc_link_rest<<<tgrid, GG_TILE_NT, 0, C.s>>>(g->out_off, g->out_adj, t->coord, t->ntiles, V, rounds, skip,
                                                      C.comp, C.f);
        C.launches++;
        if (use_in)
        {
            gg_tiles *ti = nullptr;
            GG_CHECK(gg_tiles_get(g, 1, C.s, &ti));
            k_cc_link_rest<<<gg_persistent_grid((const void *)k_cc_link_rest, ti->ntiles), GG_TILE_NT, 0, C.s>>>(
                g->in_off, g->in_adj, ti->coord, ti->ntiles, V, 0, skip, C.comp, C.f);
            C.launches++;
        }
        GG_CHECK(compress(C));
        GG_CHECK(mark(C));
        GG_CUDA(cudaGetLastError());
        res.iterations = rounds;
    }
    k_cc_roots<<<grid_for(V), 256, 0, C.s>>>(C.comp, V, C.f);
    C.launches++;
    GG_CUDA(cudaGetLastError());
    if (components) GG_CHECK(gg_copy_d2h(components, C.comp, (size_t)V * 4, C.s));
    GG_CHECK(read_flags(C));
    res.components = C.h->roots;
    res.launches = C.launches;
    if (C.profile)
        for (size_t i = 0; i + 1 < C.evs.size(); i += 2) res.kernel_ms += gg_event_ms(C.evs[i], C.evs[i + 1]);
    if (r) *r = res;
    return GG_OK;
}

extern "C" gg_status gg_cc_device_labels(const gg_graph *g, const uint32_t **components)
{
    if (!g || !g->work[0].ptr) return gg_fail(GG_ERR_INVALID, "no connected-components run on this mapping");
    if (components) *components = (const uint32_t *)g->work[0].ptr;
    return GG_OK;
}
