/*
 * CSR and CSC built on the device from an edge list.
 *
 * The reference builds its CSR with the OpenGraph pair sortRunAlgorithms +
 * graphCSRAssignEdgeList (call sites SSSP.c:552-565, bellmanFord.c:737-744;
 * the OpenGraph sources are absent from the snapshot).  The host build here,
 * graphCSRFromEdgeList, sorts the words (key << b | neighbour) with a stable
 * LSD radix sort (b = bits for V), so each row lists its neighbours in
 * ascending id and duplicate edges keep their input order.  This file sorts
 * the same words the same way on the GPU, so every array it produces is
 * identical to the host build's:
 *
 *   k_make_keys   (src << b | dst) for the CSR or (dst << b | src) for the
 *                 CSC, with the edge weight as payload; ids >= V flagged
 *   per 8-bit digit, least significant first (2b bits in all):
 *     k_rdx_count    per-tile digit counts, digit-major (counts[d][tile])
 *     scan           exclusive scan of the counts: the first output slot of
 *                    every (digit, tile), in digit-then-tile order
 *     k_rdx_scatter  stable rank within the tile (per-warp digit counters
 *                    and __match_any_sync), the tile reordered by digit in
 *                    shared memory, then written out in runs
 *   k_split       neighbour ids, row offsets from the row boundaries, and
 *                 the out-degrees
 *
 * A pass reads the keys twice and writes them once (the reduce-then-scan
 * form: no block waits on another).  Tiles are 4096 keys (256 threads x 16).
 */
#include <cuda_runtime.h>

#include <cstring>
#include <utility>

#include "gg_internal.h"

namespace {

constexpr int RDX_BINS = 256;
constexpr int RDX_THREADS = 256;
constexpr int RDX_ITEMS = 16;
constexpr int RDX_TILE = RDX_THREADS * RDX_ITEMS;
constexpr int RDX_WARPS = RDX_THREADS / 32;

constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_CHUNK = SCAN_THREADS * SCAN_ITEMS;
constexpr int SCAN_TOP_ITEMS = 64; /* the single-block pass scans up to 65536 chunk sums */

__device__ __forceinline__ uint32_t digit_of(uint64_t k, int shift) { return (uint32_t)(k >> shift) & (RDX_BINS - 1); }

/* an id that cannot collide with a digit: invalid lanes match only themselves */
__device__ __forceinline__ uint32_t match_key(bool valid, uint32_t d, uint32_t lane) { return valid ? d : RDX_BINS + lane; }

__global__ void k_make_keys(const uint32_t *__restrict__ key, const uint32_t *__restrict__ other,
                            const float *__restrict__ w, uint64_t n, uint32_t V, int b, uint64_t *out, float *wout,
                            uint32_t *bad)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    {
        const uint32_t k = key[i], o = other[i];
        if (k >= V || o >= V) atomicOr(bad, 1u);
        out[i] = ((uint64_t)k << b) | o;
        if (w) wout[i] = w[i];
    }
}

/* tile elements: warp w takes the 32 * RDX_ITEMS consecutive keys from
 * tile base + w * 32 * RDX_ITEMS, lane-interleaved per step; the same map
 * in both kernels */
__global__ void __launch_bounds__(RDX_THREADS) k_rdx_count(const uint64_t *__restrict__ keys, uint64_t n, int shift,
                                                           uint32_t ntiles, uint32_t *counts)
{
    __shared__ uint32_t h[RDX_WARPS][RDX_BINS];
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5, tile = blockIdx.x;
    for (int i = threadIdx.x; i < RDX_WARPS * RDX_BINS; i += RDX_THREADS) (&h[0][0])[i] = 0u;
    __syncthreads();
    const uint64_t base = (uint64_t)tile * RDX_TILE + (uint64_t)w * 32 * RDX_ITEMS + lane;
    uint64_t k[RDX_ITEMS];
#pragma unroll
    for (int it = 0; it < RDX_ITEMS; it++)
    {
        const uint64_t i = base + (uint64_t)it * 32;
        k[it] = i < n ? keys[i] : 0ull;
    }
#pragma unroll
    for (int it = 0; it < RDX_ITEMS; it++)
    {
        const bool valid = base + (uint64_t)it * 32 < n;
        const uint32_t d = digit_of(k[it], shift);
        const uint32_t peers = __match_any_sync(0xffffffffu, match_key(valid, d, lane));
        /* one lane per digit group adds it: bins of one warp have one writer */
        if (valid && (peers & ((1u << lane) - 1u)) == 0u) h[w][d] += (uint32_t)__popc(peers);
        __syncwarp();
    }
    __syncthreads();
    uint32_t t = 0;
#pragma unroll
    for (int ww = 0; ww < RDX_WARPS; ww++) t += h[ww][threadIdx.x];
    counts[(size_t)threadIdx.x * ntiles + tile] = t;
}

constexpr int SCATTER_SMEM = RDX_TILE * 12 + RDX_WARPS * RDX_BINS * 4 + 2 * RDX_BINS * 4 + RDX_WARPS * 4;

__global__ void __launch_bounds__(RDX_THREADS) k_rdx_scatter(const uint64_t *__restrict__ keys,
                                                             const float *__restrict__ pay, uint64_t n, int shift,
                                                             uint32_t ntiles, const uint32_t *__restrict__ first,
                                                             uint64_t *__restrict__ okeys, float *__restrict__ opay)
{
    /* dynamic shared memory, SCATTER_SMEM bytes: the tile's keys and
     * payload in digit order, per-warp digit counts (then their exclusive
     * prefix over warps), each digit's first output slot and its tile-local
     * start, the warp totals of the digit scan */
    extern __shared__ __align__(16) unsigned char smem[];
    uint64_t *skey = reinterpret_cast<uint64_t *>(smem);
    float *spay = reinterpret_cast<float *>(smem + RDX_TILE * 8);
    uint32_t(*wcnt)[RDX_BINS] = reinterpret_cast<uint32_t(*)[RDX_BINS]>(smem + RDX_TILE * 12);
    uint32_t *gfirst = reinterpret_cast<uint32_t *>(smem + RDX_TILE * 12 + RDX_WARPS * RDX_BINS * 4);
    uint32_t *tstart = gfirst + RDX_BINS;
    uint32_t *wtot = tstart + RDX_BINS;
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5, tile = blockIdx.x;
    for (int i = threadIdx.x; i < RDX_WARPS * RDX_BINS; i += RDX_THREADS) (&wcnt[0][0])[i] = 0u;
    gfirst[threadIdx.x] = first[(size_t)threadIdx.x * ntiles + tile];
    __syncthreads();
    const uint64_t base = (uint64_t)tile * RDX_TILE + (uint64_t)w * 32 * RDX_ITEMS + lane;
    uint64_t k[RDX_ITEMS];
    uint32_t rank[RDX_ITEMS];
#pragma unroll
    for (int it = 0; it < RDX_ITEMS; it++)
    {
        const uint64_t i = base + (uint64_t)it * 32;
        k[it] = i < n ? keys[i] : 0ull;
    }
    /* rank among the warp's earlier keys of the same digit, in element order */
#pragma unroll
    for (int it = 0; it < RDX_ITEMS; it++)
    {
        const bool valid = base + (uint64_t)it * 32 < n;
        const uint32_t d = digit_of(k[it], shift);
        const uint32_t peers = __match_any_sync(0xffffffffu, match_key(valid, d, lane));
        const uint32_t before = (uint32_t)__popc(peers & ((1u << lane) - 1u));
        const uint32_t seen = valid ? wcnt[w][d] : 0u;
        __syncwarp();
        if (valid && before == 0u) wcnt[w][d] = seen + (uint32_t)__popc(peers);
        __syncwarp();
        rank[it] = seen + before;
    }
    __syncthreads();
    /* thread t = digit t: exclusive prefix over warps, then the tile's
     * digit starts by a block scan of the digit totals */
    uint32_t run = 0;
#pragma unroll
    for (int ww = 0; ww < RDX_WARPS; ww++)
    {
        const uint32_t c = wcnt[ww][threadIdx.x];
        wcnt[ww][threadIdx.x] = run;
        run += c;
    }
    uint32_t incl = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += y;
    }
    if (lane == 31) wtot[w] = incl;
    __syncthreads();
    uint32_t wbase = 0;
    for (uint32_t ww = 0; ww < w; ww++) wbase += wtot[ww];
    tstart[threadIdx.x] = wbase + incl - run;
    __syncthreads();
    /* the tile in digit order in shared memory */
#pragma unroll
    for (int it = 0; it < RDX_ITEMS; it++)
    {
        const uint64_t i = base + (uint64_t)it * 32;
        if (i < n)
        {
            const uint32_t d = digit_of(k[it], shift);
            const uint32_t at = tstart[d] + wcnt[w][d] + rank[it];
            skey[at] = k[it];
            if (pay) spay[at] = pay[i];
        }
    }
    __syncthreads();
    /* runs of one digit go to consecutive output slots */
    const uint64_t t0 = (uint64_t)tile * RDX_TILE;
    const uint32_t cnt = (uint32_t)(n - t0 < (uint64_t)RDX_TILE ? n - t0 : (uint64_t)RDX_TILE);
    for (uint32_t j = threadIdx.x; j < cnt; j += RDX_THREADS)
    {
        const uint64_t key = skey[j];
        const uint32_t d = digit_of(key, shift);
        const uint32_t at = gfirst[d] + (j - tstart[d]);
        okeys[at] = key;
        if (pay) opay[at] = spay[j];
    }
}

/* ---- exclusive scan of a uint32 array (sums stay below 2^32) ---- */

/* block-wide exclusive scan of SCAN_CHUNK values held SCAN_ITEMS per thread;
 * returns this thread's exclusive base and the chunk total in *total */
__device__ __forceinline__ uint32_t block_scan_base(uint32_t mine, uint32_t *total)
{
    __shared__ uint32_t ws[SCAN_THREADS / 32];
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t incl = mine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += y;
    }
    if (lane == 31) ws[w] = incl;
    __syncthreads();
    static_assert(SCAN_THREADS == 1024, "one warp scans the 32 warp totals");
    if (w == 0)
    {
        const uint32_t v = ws[lane];
        uint32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        ws[lane] = x - v;
        if (lane == 31) *total = x;
    }
    __syncthreads();
    const uint32_t r = ws[w] + incl - mine;
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(const uint32_t *__restrict__ a, uint64_t m, uint32_t *sums)
{
    const uint64_t base = (uint64_t)blockIdx.x * SCAN_CHUNK + (uint64_t)threadIdx.x * SCAN_ITEMS;
    uint32_t t = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++)
        if (base + k < m) t += a[base + k];
    __shared__ uint32_t tot;
    block_scan_base(t, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

/* one block: exclusive scan of the chunk sums in place (nb <= 65536) */
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_top(uint32_t *sums, uint32_t nb)
{
    const uint32_t base = threadIdx.x * SCAN_TOP_ITEMS;
    uint32_t v[SCAN_TOP_ITEMS], t = 0;
#pragma unroll
    for (int k = 0; k < SCAN_TOP_ITEMS; k++)
    {
        v[k] = base + k < nb ? sums[base + k] : 0u;
        t += v[k];
    }
    __shared__ uint32_t tot;
    uint32_t run = block_scan_base(t, &tot);
#pragma unroll
    for (int k = 0; k < SCAN_TOP_ITEMS; k++)
        if (base + k < nb)
        {
            sums[base + k] = run;
            run += v[k];
        }
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_down(uint32_t *a, uint64_t m, const uint32_t *__restrict__ sums)
{
    const uint64_t base = (uint64_t)blockIdx.x * SCAN_CHUNK + (uint64_t)threadIdx.x * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS], t = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++)
    {
        v[k] = base + k < m ? a[base + k] : 0u;
        t += v[k];
    }
    __shared__ uint32_t tot;
    uint32_t run = sums[blockIdx.x] + block_scan_base(t, &tot);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++)
        if (base + k < m)
        {
            a[base + k] = run;
            run += v[k];
        }
}

/* neighbour ids, and off[v] = the first slot whose key is >= v (off[V] = n):
 * slot i writes the offsets of the rows between its predecessor's key and
 * its own */
__global__ void k_split(const uint64_t *__restrict__ keys, uint64_t n, int b, uint32_t V, uint32_t *off, uint32_t *adj,
                        const float *__restrict__ pay, float *wout)
{
    const uint64_t mask = (1ull << b) - 1ull;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += (uint64_t)gridDim.x * blockDim.x)
    {
        const int64_t prev = i ? (int64_t)(keys[i - 1] >> b) : -1;
        int64_t cur = i < n ? (int64_t)(keys[i] >> b) : (int64_t)V;
        if (cur > (int64_t)V) cur = V; /* only an id >= V (reported) gets here */
        for (int64_t v = prev + 1; v <= cur; v++) off[v] = (uint32_t)i;
        if (i < n)
        {
            adj[i] = (uint32_t)(keys[i] & mask);
            if (wout) wout[i] = pay[i];
        }
    }
}

__global__ void k_degrees(const uint32_t *__restrict__ off, uint32_t V, uint32_t *deg)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
        deg[v] = off[v + 1] - off[v];
}

/* largest weight above 0 (0 when none), as the edge-list readers record it */
__global__ void k_max_weight(const float *__restrict__ w, uint64_t n, unsigned int *out)
{
    float m = 0.0f;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        if (w[i] > m) m = w[i];
    if (m > 0.0f) atomicMax(out, __float_as_uint(m)); /* positive floats order as their bits */
}

int bits_for(uint32_t V)
{
    int b = 1;
    while (b < 32 && (1ull << b) < V) b++;
    return b;
}

int grid_for(uint64_t n, int threads)
{
    const uint64_t b = (n + threads - 1) / threads, cap = (uint64_t)gg_sm_count() * 8;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

struct SortBufs
{
    uint64_t *keys, *tmp;
    float *pay, *ptmp; /* null when unweighted */
    uint32_t *counts, *sums;
};

/* stable LSD sort of n words on their low `bits` bits; the sorted words
 * (and payload) end in B.keys / B.pay */
gg_status radix_sort(SortBufs &B, uint64_t n, int bits, cudaStream_t s)
{
    if (n <= 1) return GG_OK;
    static bool attr_set = false; /* one device per process */
    if (!attr_set)
    {
        GG_CUDA(cudaFuncSetAttribute(k_rdx_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, SCATTER_SMEM));
        attr_set = true;
    }
    const uint32_t ntiles = (uint32_t)((n + RDX_TILE - 1) / RDX_TILE);
    const uint64_t m = (uint64_t)RDX_BINS * ntiles;
    const uint32_t nb = (uint32_t)((m + SCAN_CHUNK - 1) / SCAN_CHUNK);
    if (nb > (uint32_t)SCAN_THREADS * SCAN_TOP_ITEMS) return gg_fail(GG_ERR_INVALID, "edge list too long to sort");
    for (int shift = 0; shift < bits; shift += 8)
    {
        k_rdx_count<<<ntiles, RDX_THREADS, 0, s>>>(B.keys, n, shift, ntiles, B.counts);
        k_scan_reduce<<<nb, SCAN_THREADS, 0, s>>>(B.counts, m, B.sums);
        k_scan_top<<<1, SCAN_THREADS, 0, s>>>(B.sums, nb);
        k_scan_down<<<nb, SCAN_THREADS, 0, s>>>(B.counts, m, B.sums);
        k_rdx_scatter<<<ntiles, RDX_THREADS, SCATTER_SMEM, s>>>(B.keys, B.pay, n, shift, ntiles, B.counts, B.tmp, B.ptmp);
        GG_CUDA(cudaGetLastError());
        std::swap(B.keys, B.tmp);
        std::swap(B.pay, B.ptmp);
    }
    return GG_OK;
}

/* one direction: rows keyed by `key`, neighbours from `other` */
gg_status build_direction(gg_graph *g, SortBufs &B, const uint32_t *key, const uint32_t *other, const float *w,
                          uint32_t **off, uint32_t **adj, float **wout, uint32_t *bad, cudaStream_t s)
{
    const uint32_t V = g->V, E = g->E;
    const int b = bits_for(V);
    k_make_keys<<<grid_for(E, 256), 256, 0, s>>>(key, other, w, E, V, b, B.keys, B.pay, bad);
    GG_CUDA(cudaGetLastError());
    GG_CHECK(radix_sort(B, E, 2 * b, s));
    GG_CHECK(gg_dev_alloc(g, (void **)off, ((size_t)V + 1) * 4));
    GG_CHECK(gg_dev_alloc(g, (void **)adj, ((size_t)E + GG_EDGE_PAD) * 4));
    GG_CUDA(cudaMemsetAsync(*adj + E, 0, GG_EDGE_PAD * 4, s));
    if (wout)
    {
        GG_CHECK(gg_dev_alloc(g, (void **)wout, ((size_t)E + GG_EDGE_PAD) * 4));
        GG_CUDA(cudaMemsetAsync(*wout + E, 0, GG_EDGE_PAD * 4, s));
    }
    k_split<<<grid_for((uint64_t)E + 1, 256), 256, 0, s>>>(B.keys, E, b, V, *off, *adj, B.pay, wout ? *wout : nullptr);
    GG_CUDA(cudaGetLastError());
    return GG_OK;
}

} // namespace

gg_status gg_build_arrays(gg_graph *g, const uint32_t *src, const uint32_t *dst, const float *w, uint32_t what,
                          cudaStream_t s)
{
    const uint32_t V = g->V, E = g->E;
    if (V == 0) return gg_fail(GG_ERR_INVALID, "a graph needs at least one vertex");
    /* weights given and asked for; without given weights a _W request gets
     * the reference's constant 0.0001f, as gg_graph_map does */
    const bool weighted = w != nullptr && (what & (GG_MAP_OUT_W | GG_MAP_IN_W));
    SortBufs B{};
    void *bad = nullptr;
    const uint64_t ntiles = ((uint64_t)E + RDX_TILE - 1) / RDX_TILE;
    const uint64_t m = (uint64_t)RDX_BINS * (ntiles ? ntiles : 1);
    gg_status st = GG_OK;
    do
    {
        if ((st = gg_dev_alloc(g, (void **)&B.keys, (size_t)E * 8 + 16)) != GG_OK) break;
        if ((st = gg_dev_alloc(g, (void **)&B.tmp, (size_t)E * 8 + 16)) != GG_OK) break;
        if (weighted)
        {
            if ((st = gg_dev_alloc(g, (void **)&B.pay, (size_t)E * 4 + 16)) != GG_OK) break;
            if ((st = gg_dev_alloc(g, (void **)&B.ptmp, (size_t)E * 4 + 16)) != GG_OK) break;
        }
        if ((st = gg_dev_alloc(g, (void **)&B.counts, (size_t)m * 4)) != GG_OK) break;
        if ((st = gg_dev_alloc(g, (void **)&B.sums, ((m + SCAN_CHUNK - 1) / SCAN_CHUNK) * 4 + 16)) != GG_OK) break;
        if ((st = gg_dev_alloc(g, &bad, 16)) != GG_OK) break;
        if (cudaMemsetAsync(bad, 0, 16, s) != cudaSuccess)
        {
            st = gg_fail(GG_ERR_CUDA, "cudaMemsetAsync");
            break;
        }
        const float *wp = weighted ? w : nullptr;
        const bool need_out = what & (GG_MAP_OUT | GG_MAP_OUT_W), need_in = what & (GG_MAP_IN | GG_MAP_IN_W);
        /* the CSR is always built: the out-degrees come from it */
        SortBufs F = B;
        if ((st = build_direction(g, F, src, dst, wp, &g->out_off, &g->out_adj,
                                  (weighted && (what & GG_MAP_OUT_W)) ? &g->out_w : nullptr, (uint32_t *)bad, s)) != GG_OK)
            break;
        if ((st = gg_dev_alloc(g, (void **)&g->out_deg, (size_t)V * 4 + 16)) != GG_OK) break;
        k_degrees<<<grid_for(V, 256), 256, 0, s>>>(g->out_off, V, g->out_deg);
        if (need_in)
        {
            SortBufs I = B;
            if ((st = build_direction(g, I, dst, src, wp, &g->in_off, &g->in_adj,
                                      (weighted && (what & GG_MAP_IN_W)) ? &g->in_w : nullptr, (uint32_t *)bad, s)) != GG_OK)
                break;
        }
        if (!need_out)
        {
            /* the CSR was only the degree source */
            const size_t off_bytes = ((size_t)V + 1) * 4, edge_alloc = ((size_t)E + GG_EDGE_PAD) * 4;
            if (cudaStreamSynchronize(s) != cudaSuccess)
            {
                st = gg_fail(GG_ERR_CUDA, "cudaStreamSynchronize");
                break;
            }
            gg_dev_free(g, g->out_off, off_bytes);
            gg_dev_free(g, g->out_adj, edge_alloc);
            g->out_off = nullptr;
            g->out_adj = nullptr;
        }
        unsigned int flags[2] = {0u, 0u};
        if (cudaMemcpyAsync(flags, bad, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        {
            st = gg_fail(GG_ERR_CUDA, "cudaMemcpyAsync");
            break;
        }
        if ((st = gg_wait(s)) != GG_OK) break;
        if (flags[0]) st = gg_fail(GG_ERR_INVALID, "edge list has a vertex id >= num_vertices");
        if (weighted && st == GG_OK)
        {
            /* the largest weight, for the host copy's max_weight */
            unsigned int *mx = (unsigned int *)bad + 1;
            cudaMemsetAsync(mx, 0, 4, s);
            k_max_weight<<<grid_for(E, 256), 256, 0, s>>>(w, E, mx);
            unsigned int bits = 0;
            cudaMemcpyAsync(&bits, mx, 4, cudaMemcpyDeviceToHost, s);
            if ((st = gg_wait(s)) == GG_OK) memcpy(&g->max_weight, &bits, 4);
        }
    } while (false);
    gg_wait(s);
    gg_dev_free(g, B.keys, (size_t)E * 8 + 16);
    gg_dev_free(g, B.tmp, (size_t)E * 8 + 16);
    gg_dev_free(g, B.pay, (size_t)E * 4 + 16);
    gg_dev_free(g, B.ptmp, (size_t)E * 4 + 16);
    gg_dev_free(g, B.counts, (size_t)m * 4);
    gg_dev_free(g, B.sums, ((m + SCAN_CHUNK - 1) / SCAN_CHUNK) * 4 + 16);
    gg_dev_free(g, bad, 16);
    if (st == GG_OK && !weighted)
    {
        if (what & GG_MAP_OUT_W) st = gg_fill_constant_weights(g, &g->out_w, E, s);
        if (st == GG_OK && (what & GG_MAP_IN_W)) st = gg_fill_constant_weights(g, &g->in_w, E, s);
        if (st == GG_OK) st = gg_wait(s);
    }
    if (st == GG_OK) g->what = what | (g->in_off ? GG_MAP_IN : 0u) | (g->out_off ? GG_MAP_OUT : 0u);
    return st;
}
