/*
 * Hot-vertex table of the pull gather: the GPU counterpart of the reference
 * FPGA's vertex cache (cu_vertex_cache_reuse_control.sv keeps frequently
 * read vertices on chip, marked through heat bits that EXTRACT_VALUE masks
 * off the neighbour ids).  Here the H vertices with the most out-edges -- the
 * contributions a pull gather reads most often -- get slots 0..H-1, and a
 * copy of the CSC neighbour ids carries them as 0x80000000 | slot, so a
 * gather kernel can serve those reads from a table in shared memory filled
 * once per launch.  On R-MAT graphs in natural order the 16K hottest of 16.7M
 * vertices receive 30% of all gathers, and their sectors sit on a few L2
 * slices that otherwise saturate first.
 *
 * Preparation, once per mapping: a histogram of out-degrees (clamped at
 * 65535) read back to the host gives the threshold degree T; vertices above
 * T and, up to H, vertices at T take slots by atomics (which of the ties win
 * does not matter: the table holds exact copies); one pass over the CSC
 * writes the encoded ids.
 */
#include <cuda_runtime.h>

#include <vector>

#include "gg_internal.h"

namespace {

constexpr uint32_t NO_SLOT = 0xffffffffu;

/* out-degree histogram (clamped at 65535): degrees below 4096 -- nearly all
 * of them on skewed graphs, so global atomics on those bins would serialise
 * -- are counted in shared memory per CTA and flushed once */
__global__ void __launch_bounds__(256) k_deg_hist(const uint32_t *__restrict__ outdeg, uint32_t V, uint32_t *hist)
{
    constexpr uint32_t LOW = 4096;
    __shared__ uint32_t s[LOW];
    for (uint32_t i = threadIdx.x; i < LOW; i += blockDim.x) s[i] = 0;
    __syncthreads();
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
    {
        const uint32_t d = min(outdeg[v], 65535u);
        if (d < LOW)
            atomicAdd(&s[d], 1u);
        else
            atomicAdd(&hist[d], 1u);
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < LOW; i += blockDim.x)
        if (s[i]) atomicAdd(&hist[i], s[i]);
}

__global__ void k_hot_mark(const uint32_t *__restrict__ outdeg, uint32_t V, uint32_t T, uint32_t above,
                           uint32_t H, uint32_t *slot_of, uint32_t *hot_list, uint32_t *counters)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
    {
        const uint32_t d = min(outdeg[v], 65535u);
        uint32_t slot = NO_SLOT;
        if (d > T)
            slot = atomicAdd(&counters[0], 1u);
        else if (d == T && T > 0)
        {
            const uint32_t k = atomicAdd(&counters[1], 1u);
            if (above + k < H) slot = above + k;
        }
        slot_of[v] = slot;
        if (slot != NO_SLOT) hot_list[slot] = v;
    }
}

/* ids -> encoded ids.  Every CTA first puts the hot vertices into a Bloom
 * filter in shared memory (BLOOM_BITS bits, two hashes): an id whose two
 * bits are not both set is not hot and is copied as it is, and only the
 * others (the hot ones, ~22% of the edges of R-MAT-24, and rare false
 * positives) read their slot.  Reading the slot of every id at random had
 * made the pass ~0.9 ms of L2 requests at R-MAT-24.  The ids stream in
 * 16-byte loads, four in flight per thread. */
constexpr uint32_t BLOOM_BITS = 1u << 19; /* 64 KB */

__device__ __forceinline__ uint32_t bloom_h1(uint32_t u) { return (u * 0x9E3779B1u) >> 13; }
__device__ __forceinline__ uint32_t bloom_h2(uint32_t u) { return (u * 0x85EBCA77u + 0x165667B1u) >> 13; }

__global__ void __launch_bounds__(1024) k_hot_encode(const uint32_t *__restrict__ adj, uint64_t n,
                                                     const uint32_t *__restrict__ slot_of,
                                                     const uint32_t *__restrict__ hot_list,
                                                     const uint32_t *__restrict__ counters, uint32_t H,
                                                     uint32_t *__restrict__ out)
{
    extern __shared__ uint32_t bloom[];
    for (uint32_t i = threadIdx.x; i < BLOOM_BITS / 32; i += blockDim.x) bloom[i] = 0u;
    __syncthreads();
    const uint32_t taken = counters[0] + counters[1];
    const uint32_t nh = taken < H ? taken : H;
    for (uint32_t i = threadIdx.x; i < nh; i += blockDim.x)
    {
        const uint32_t u = hot_list[i], b1 = bloom_h1(u), b2 = bloom_h2(u);
        atomicOr(&bloom[b1 >> 5], 1u << (b1 & 31));
        atomicOr(&bloom[b2 >> 5], 1u << (b2 & 31));
    }
    __syncthreads();
    auto enc = [&](uint32_t u) -> uint32_t {
        const uint32_t b1 = bloom_h1(u), b2 = bloom_h2(u);
        if (!((bloom[b1 >> 5] >> (b1 & 31)) & (bloom[b2 >> 5] >> (b2 & 31)) & 1u)) return u;
        const uint32_t sl = slot_of[u];
        return sl == NO_SLOT ? u : (GG_HOT_FLAG | sl);
    };
    const uint64_t nv = n / 4, stride = (uint64_t)gridDim.x * blockDim.x;
    const uint4 *a4 = reinterpret_cast<const uint4 *>(adj);
    uint4 *o4 = reinterpret_cast<uint4 *>(out);
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    for (; i + 3 * stride < nv; i += 4 * stride)
    {
        uint4 v[4];
#pragma unroll
        for (int k = 0; k < 4; k++) v[k] = __ldcs(a4 + i + k * stride);
#pragma unroll
        for (int k = 0; k < 4; k++)
        {
            v[k].x = enc(v[k].x);
            v[k].y = enc(v[k].y);
            v[k].z = enc(v[k].z);
            v[k].w = enc(v[k].w);
            o4[i + k * stride] = v[k];
        }
    }
    for (; i < nv; i += stride)
    {
        uint4 v = __ldcs(a4 + i);
        v.x = enc(v.x);
        v.y = enc(v.y);
        v.z = enc(v.z);
        v.w = enc(v.w);
        o4[i] = v;
    }
    /* the last n % 4 ids */
    if (blockIdx.x == 0 && threadIdx.x < n - nv * 4)
    {
        const uint64_t e = nv * 4 + threadIdx.x;
        out[e] = enc(adj[e]);
    }
}

} // namespace

gg_status gg_hot_prepare(gg_graph *g, cudaStream_t s, uint32_t cap)
{
    if (!g->in_adj || !g->out_deg) return gg_fail(GG_ERR_INVALID, "the hot-vertex table needs GG_MAP_IN");
    const uint32_t V = g->V, E = g->E;
    if (V >= GG_HOT_FLAG) return gg_fail(GG_ERR_INVALID, "graph too large for flag-encoded ids");
    if (cap < 1 || cap > GG_HOT_ENTRIES) return gg_fail(GG_ERR_INVALID, "hot table capacity out of range");
    gg_tiles &t = g->hot_tiles;
    if (!t.coord)
    {
        const uint32_t items = 32u * GG_HOT_IPT;
        const uint64_t nt = ((uint64_t)V + E + items - 1) / items;
        if (nt >= 0xffffffffull) return gg_fail(GG_ERR_INVALID, "graph too large for 32-bit tile ids");
        t.ntiles = (uint32_t)(nt ? nt : 1);
        GG_CHECK(gg_dev_alloc(g, (void **)&t.coord, ((size_t)t.ntiles + 1) * sizeof(uint2)));
        GG_CHECK(gg_launch_tile_coords(g->in_off, V, E, t.ntiles, t.coord, s, items));
    }
    if (g->hot_adj && g->hot_cap == cap) return GG_OK;
    const uint32_t H = V < cap ? V : cap;
    void *hist, *slot_of, *cnt;
    GG_CHECK(gg_work(g, 25, 65536 * 4, &hist));
    GG_CHECK(gg_work(g, 26, (size_t)V * 4, &slot_of));
    GG_CHECK(gg_work(g, 27, 16, &cnt));
    GG_CUDA(cudaMemsetAsync(hist, 0, 65536 * 4, s));
    GG_CUDA(cudaMemsetAsync(cnt, 0, 16, s));
    const int grid = gg_sm_count() * 8;
    k_deg_hist<<<gg_sm_count() * 2, 256, 0, s>>>(g->out_deg, V, (uint32_t *)hist);
    GG_CUDA(cudaGetLastError());
    std::vector<uint32_t> h(65536);
    GG_CHECK(gg_wait(s)); /* bounded, before a copy to pageable memory */
    GG_CUDA(cudaMemcpyAsync(h.data(), hist, 65536 * 4, cudaMemcpyDeviceToHost, s));
    GG_CHECK(gg_wait(s));
    /* threshold: the degree T with fewer than H vertices above it */
    uint32_t above = 0, T = 0;
    for (int d = 65535; d >= 0; d--)
    {
        if (above + h[d] >= H || d == 0)
        {
            T = (uint32_t)d;
            break;
        }
        above += h[d];
    }
    if (!g->hot_list) GG_CHECK(gg_dev_alloc(g, (void **)&g->hot_list, (size_t)GG_HOT_ENTRIES * 4));
    if (!g->hot_adj) GG_CHECK(gg_dev_alloc(g, (void **)&g->hot_adj, ((size_t)E + GG_EDGE_PAD) * 4));
    k_hot_mark<<<grid, 256, 0, s>>>(g->out_deg, V, T, above, H, (uint32_t *)slot_of, g->hot_list, (uint32_t *)cnt);
    /* one CTA of 1024 threads per SM (60 registers a thread); adj and out are
     * whole allocations, 16-byte aligned for the vector loads */
    GG_CUDA(cudaFuncSetAttribute(k_hot_encode, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(BLOOM_BITS / 8)));
    k_hot_encode<<<gg_sm_count(), 1024, BLOOM_BITS / 8, s>>>(g->in_adj, (uint64_t)E, (const uint32_t *)slot_of,
                                                              g->hot_list, (const uint32_t *)cnt, H, g->hot_adj);
    GG_CUDA(cudaGetLastError());
    std::vector<uint32_t> c(4);
    GG_CHECK(gg_wait(s));
    GG_CUDA(cudaMemcpyAsync(c.data(), cnt, 16, cudaMemcpyDeviceToHost, s));
    GG_CHECK(gg_wait(s));
    g->hot_n = T > 0 ? (c[0] + (c[1] < H - above ? c[1] : H - above)) : c[0];
    if (g->hot_n > H) g->hot_n = H;
    g->hot_cap = cap;
    return GG_OK;
}
