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
 *     k_rdx_count    per-tile digit counts, tile-major (counts[tile][d]), by
 *                    shared atomics (one per warp when its keys share a digit)
 *     column scan    k_col_reduce / k_col_top / k_col_down: counts[tile][d]
 *                    becomes the first output slot of digit d's keys of that
 *                    tile (keys of smaller digits, then of digit d in
 *                    earlier tiles); every access is a coalesced row
 *     k_rdx_scatter  stable rank within the tile (per-warp digit counters;
 *                    lanes with equal digits found by eight ballots), the
 *                    tile reordered by digit in shared memory, then written
 *                    out in runs
 *   k_split       neighbour ids, row offsets from the row boundaries, and
 *                 the out-degrees
 *   the CSC: k_swap_fields turns the CSR's sorted words into
 *                 (dst << b | src) in (src, dst) order, and a stable sort of
 *                 the dst field alone finishes it (b/8 passes, not 2b/8)
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

constexpr int COL_TILES = 64; /* tiles per block of the column scan */

__device__ __forceinline__ uint32_t digit_of(uint64_t k, int shift) { return (uint32_t)(k >> shift) & (RDX_BINS - 1); }

/* lanes of the warp holding a valid key with the same digit (warp
 * multisplit: one ballot per digit bit, ALU work instead of a match
 * instruction); meaningful for valid lanes only */
__device__ __forceinline__ uint32_t digit_peers(bool valid, uint32_t d)
{
    uint32_t m = __ballot_sync(0xffffffffu, valid);
#pragma unroll
    for (int b = 0; b < 8; b++)
    {
        const uint32_t bit = (d >> b) & 1u;
        const uint32_t v = __ballot_sync(0xffffffffu, bit);
        m &= bit ? v : ~v;
    }
    return m;
}

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
    __shared__ uint32_t h[RDX_BINS];
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5, tile = blockIdx.x;
    h[threadIdx.x] = 0u;
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
        /* a warp whose keys all share one digit (frequent in the skewed
         * high digits of row ids) adds 32 at once; otherwise every key adds
         * itself */
        /* every lane takes part in the shuffle and the vote */
        const uint32_t d0 = __shfl_sync(0xffffffffu, d, 0);
        if (__all_sync(0xffffffffu, valid && d == d0))
        {
            if (lane == 0) atomicAdd(&h[d], 32u);
        }
        else if (valid)
            atomicAdd(&h[d], 1u);
    }
    __syncthreads();
    counts[(size_t)tile * RDX_BINS + threadIdx.x] = h[threadIdx.x];
}

constexpr int SCATTER_SMEM = RDX_TILE * 12 + RDX_WARPS * RDX_BINS * 4 + 2 * RDX_BINS * 4 + RDX_WARPS * 4;

__global__ void __launch_bounds__(RDX_THREADS, 3) k_rdx_scatter(const uint64_t *__restrict__ keys,
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
    gfirst[threadIdx.x] = first[(size_t)tile * RDX_BINS + threadIdx.x];
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
    /* rank among the warp's earlier keys of the same digit, in element
     * order: the group's lowest lane advances the warp's digit counter by
     * the group size and hands the old value to its peers */
#pragma unroll
    for (int it = 0; it < RDX_ITEMS; it++)
    {
        const bool valid = base + (uint64_t)it * 32 < n;
        const uint32_t d = digit_of(k[it], shift);
        const uint32_t peers = digit_peers(valid, d);
        const uint32_t before = (uint32_t)__popc(peers & ((1u << lane) - 1u));
        const int leader = valid ? __ffs(peers) - 1 : (int)lane;
        uint32_t seen = 0;
        if (valid && before == 0u) seen = atomicAdd(&wcnt[w][d], (uint32_t)__popc(peers));
        seen = __shfl_sync(0xffffffffu, seen, leader);
        rank[it] = seen + before;
        __syncwarp();
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

/* ---- column scan of the [tile][digit] counts (thread = digit) ---- */

/* the column sums of each block of COL_TILES tiles (the loads of a block's
 * rows are independent: unrolled so they are in flight together) */
__global__ void __launch_bounds__(RDX_BINS) k_col_reduce(const uint32_t *__restrict__ counts, uint32_t ntiles,
                                                         uint32_t *csum)
{
    const uint32_t t0 = blockIdx.x * COL_TILES, t1 = min(t0 + COL_TILES, ntiles);
    uint32_t t = 0;
#pragma unroll 8
    for (uint32_t tile = t0; tile < t1; tile++) t += counts[(size_t)tile * RDX_BINS + threadIdx.x];
    csum[(size_t)blockIdx.x * RDX_BINS + threadIdx.x] = t;
}

/* one block of COL_TOP_SPLIT * RDX_BINS threads: csum[b][d] becomes the
 * first output slot of digit d in block b's tiles (the keys of all smaller
 * digits plus digit d in earlier blocks); each digit's blocks are split over
 * COL_TOP_SPLIT threads, combined through shared memory */
constexpr uint32_t COL_TOP_SPLIT = 4;

__global__ void __launch_bounds__(COL_TOP_SPLIT * RDX_BINS) k_col_top(uint32_t *csum, uint32_t nblocks)
{
    __shared__ uint32_t part[COL_TOP_SPLIT][RDX_BINS];
    __shared__ uint32_t wtot[RDX_BINS / 32];
    const uint32_t d = threadIdx.x % RDX_BINS, q = threadIdx.x / RDX_BINS;
    const uint32_t b0 = (uint32_t)((uint64_t)nblocks * q / COL_TOP_SPLIT);
    const uint32_t b1 = (uint32_t)((uint64_t)nblocks * (q + 1) / COL_TOP_SPLIT);
    uint32_t run = 0;
#pragma unroll 8
    for (uint32_t b = b0; b < b1; b++) run += csum[(size_t)b * RDX_BINS + d];
    part[q][d] = run;
    __syncthreads();
    /* digit d's total and the start of quarter q within it */
    uint32_t before = 0, total = 0;
    for (uint32_t k = 0; k < COL_TOP_SPLIT; k++)
    {
        if (k < q) before += part[k][d];
        total += part[k][d];
    }
    /* exclusive scan of the digit totals (the first RDX_BINS threads) */
    uint32_t base = 0;
    if (q == 0)
    {
        const uint32_t lane = d & 31, w = d >> 5;
        uint32_t incl = total;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= (uint32_t)o) incl += y;
        }
        if (lane == 31) wtot[w] = incl;
        base = incl - total;
    }
    __syncthreads();
    if (q == 0)
    {
        for (uint32_t k = 0; k < (d >> 5); k++) base += wtot[k];
        part[0][d] = base;
    }
    __syncthreads();
    uint32_t at = part[0][d] + before;
    __syncthreads();
    for (uint32_t b = b0; b < b1; b++)
    {
        const uint32_t c = csum[(size_t)b * RDX_BINS + d];
        csum[(size_t)b * RDX_BINS + d] = at;
        at += c;
    }
}

__global__ void __launch_bounds__(RDX_BINS) k_col_down(uint32_t *counts, uint32_t ntiles,
                                                       const uint32_t *__restrict__ csum)
{
    const uint32_t t0 = blockIdx.x * COL_TILES, t1 = min(t0 + COL_TILES, ntiles);
    uint32_t run = csum[(size_t)blockIdx.x * RDX_BINS + threadIdx.x];
    uint32_t tile = t0;
    /* eight rows loaded together, then their running prefix written */
    for (; tile + 8 <= t1; tile += 8)
    {
        uint32_t c[8];
#pragma unroll
        for (int k = 0; k < 8; k++) c[k] = counts[(size_t)(tile + k) * RDX_BINS + threadIdx.x];
#pragma unroll
        for (int k = 0; k < 8; k++)
        {
            counts[(size_t)(tile + k) * RDX_BINS + threadIdx.x] = run;
            run += c[k];
        }
    }
    for (; tile < t1; tile++)
    {
        uint32_t *p = counts + (size_t)tile * RDX_BINS + threadIdx.x;
        const uint32_t c = *p;
        *p = run;
        run += c;
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

/* stable LSD sort of n words on their bits lo .. bits-1 (8-bit digits from
 * bit lo up); the sorted words (and payload) end in B.keys / B.pay */
gg_status radix_sort(SortBufs &B, uint64_t n, int bits, cudaStream_t s, int lo = 0)
{
    if (n <= 1) return GG_OK;
    GG_CUDA(cudaFuncSetAttribute(k_rdx_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, SCATTER_SMEM));
    const uint32_t ntiles = (uint32_t)((n + RDX_TILE - 1) / RDX_TILE);
    const uint32_t nb = (ntiles + COL_TILES - 1) / COL_TILES;
    for (int shift = lo; shift < bits; shift += 8)
    {
        k_rdx_count<<<ntiles, RDX_THREADS, 0, s>>>(B.keys, n, shift, ntiles, B.counts);
        k_col_reduce<<<nb, RDX_BINS, 0, s>>>(B.counts, ntiles, B.sums);
        k_col_top<<<1, COL_TOP_SPLIT * RDX_BINS, 0, s>>>(B.sums, nb);
        k_col_down<<<nb, RDX_BINS, 0, s>>>(B.counts, ntiles, B.sums);
        k_rdx_scatter<<<ntiles, RDX_THREADS, SCATTER_SMEM, s>>>(B.keys, B.pay, n, shift, ntiles, B.counts, B.tmp, B.ptmp);
        GG_CUDA(cudaGetLastError());
        std::swap(B.keys, B.tmp);
        std::swap(B.pay, B.ptmp);
    }
    return GG_OK;
}

/* (row, neighbour) -> (neighbour, row) in every word */
__global__ void k_swap_fields(uint64_t *keys, uint64_t n, int b)
{
    const uint64_t mask = (1ull << b) - 1ull;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    {
        const uint64_t k = keys[i];
        keys[i] = ((k & mask) << b) | (k >> b);
    }
}

/* the sorted words of one direction -> its offsets, neighbours, weights */
gg_status split_direction(gg_graph *g, SortBufs &B, uint32_t **off, uint32_t **adj, float **wout, cudaStream_t s)
{
    const uint32_t V = g->V, E = g->E;
    const int b = bits_for(V);
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

/* the CSR: words (src << b | dst) sorted on all 2b bits */
gg_status build_csr(gg_graph *g, SortBufs &B, const uint32_t *src, const uint32_t *dst, const float *w,
                    uint32_t **off, uint32_t **adj, float **wout, uint32_t *bad, cudaStream_t s)
{
    const uint32_t V = g->V, E = g->E;
    const int b = bits_for(V);
    k_make_keys<<<grid_for(E, 256), 256, 0, s>>>(src, dst, w, E, V, b, B.keys, B.pay, bad);
    GG_CUDA(cudaGetLastError());
    GG_CHECK(radix_sort(B, E, 2 * b, s));
    return split_direction(g, B, off, adj, wout, s);
}

/* the CSC from the CSR's sorted words: with the fields swapped they are in
 * (src, dst) order, so a stable sort on the dst field alone gives
 * (dst, src) order with duplicates still in input order -- the order a
 * full sort of (dst << b | src) from the input gives -- in b/8 passes
 * instead of 2b/8 */
gg_status build_csc_from_csr(gg_graph *g, SortBufs &B, uint32_t **off, uint32_t **adj, float **wout, cudaStream_t s)
{
    const uint32_t E = g->E;
    const int b = bits_for(g->V);
    k_swap_fields<<<grid_for(E, 256), 256, 0, s>>>(B.keys, E, b);
    GG_CUDA(cudaGetLastError());
    GG_CHECK(radix_sort(B, E, 2 * b, s, b));
    return split_direction(g, B, off, adj, wout, s);
}

} // namespace

gg_status gg_build_arrays(gg_graph *g, const uint32_t *src, const uint32_t *dst, const float *w, uint32_t what,
                          cudaStream_t s)
{
    GgRange range("gg_build_csr");
    const uint32_t V = g->V, E = g->E;
    if (V == 0) return gg_fail(GG_ERR_INVALID, "a graph needs at least one vertex");
    /* weights given and asked for; without given weights a _W request gets
     * the reference's constant 0.0001f, as gg_graph_map does */
    const bool weighted = w != nullptr && (what & (GG_MAP_OUT_W | GG_MAP_IN_W));
    SortBufs B{};
    void *bad = nullptr;
    const uint64_t ntiles = ((uint64_t)E + RDX_TILE - 1) / RDX_TILE;
    const uint64_t m = (uint64_t)RDX_BINS * (ntiles ? ntiles : 1);
    const size_t sums_bytes = ((ntiles + COL_TILES - 1) / COL_TILES + 1) * RDX_BINS * 4;
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
        if ((st = gg_dev_alloc(g, (void **)&B.sums, sums_bytes)) != GG_OK) break;
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
        if ((st = build_csr(g, F, src, dst, wp, &g->out_off, &g->out_adj,
                            (weighted && (what & GG_MAP_OUT_W)) ? &g->out_w : nullptr, (uint32_t *)bad, s)) != GG_OK)
            break;
        if ((st = gg_dev_alloc(g, (void **)&g->out_deg, (size_t)V * 4 + 16)) != GG_OK) break;
        k_degrees<<<grid_for(V, 256), 256, 0, s>>>(g->out_off, V, g->out_deg);
        if (need_in)
        {
            /* F still holds the CSR's sorted words and weights */
            if ((st = build_csc_from_csr(g, F, &g->in_off, &g->in_adj,
                                         (weighted && (what & GG_MAP_IN_W)) ? &g->in_w : nullptr, s)) != GG_OK)
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
        if ((st = gg_wait(s)) != GG_OK) break; /* bounded, before a copy to pageable memory */
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
            if ((st = gg_wait(s)) != GG_OK) break;
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
    gg_dev_free(g, B.sums, sums_bytes);
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

/* ---- degree-based relabelling (the reference's -l modes) ------------------
 *
 * The reference lists its relabelling modes (README.md:362-378: 1
 * out-degree, 2 in-degree, 3 (in+out)-degree, 4/5 DBG out/in, 6/7 HUBSort
 * out/in, 8/9 HUBCluster out/in, 10 random, 11 load from file); their code is
 * in the absent OpenGraph submodule.  Each mode here is the published
 * algorithm as one sort key per vertex, (key << b) | id, sorted by the radix
 * sort above, so ties keep the original order:
 *   degree (1-3)    descending degree
 *   DBG (4/5)       degree-based grouping (Faldu et al., IISWC 2019): eight
 *                   groups, group k >= 1 holding degrees in
 *                   [avg/2 * 2^(k-1), avg/2 * 2^k) (the last one open), group
 *                   0 the rest; hotter groups first, original order inside
 *   HUBSort (6/7)   hubs (degree > avg) by descending degree, then the other
 *                   vertices in original order (Zhang et al., 2017)
 *   HUBCluster (8/9) hubs first, then the others, both in original order
 *   random (10)     SplitMix64(seed ^ id), ties by id
 * avg = E / V.  The result is label[orig] = new. */

namespace {

__global__ void k_degree_count(const uint32_t *__restrict__ ids, uint64_t n, uint32_t V, uint32_t *deg, uint32_t *bad)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    {
        const uint32_t v = ids[i];
        if (v < V)
            atomicAdd(deg + v, 1u);
        else
            atomicOr(bad, 1u);
    }
}

__device__ __forceinline__ uint64_t mode_degree(uint32_t mode, const uint32_t *dout, const uint32_t *din, uint32_t v)
{
    switch (mode)
    {
    case 1: case 4: case 6: case 8: return dout[v];
    case 2: case 5: case 7: case 9: return din[v];
    case 3: return (uint64_t)dout[v] + din[v];
    default: return 0;
    }
}

__global__ void k_degree_max(const uint32_t *__restrict__ dout, const uint32_t *__restrict__ din, uint32_t V,
                             uint32_t mode, unsigned long long *out)
{
    unsigned long long m = 0;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
    {
        const unsigned long long d = mode_degree(mode, dout, din, v);
        m = d > m ? d : m;
    }
    for (int o = 16; o > 0; o >>= 1)
    {
        const unsigned long long y = __shfl_xor_sync(0xffffffffu, m, o);
        m = y > m ? y : m;
    }
    if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}

__device__ __forceinline__ uint64_t relabel_key(uint32_t mode, uint64_t d, uint64_t dmax, uint64_t avg, uint64_t seed,
                                                uint32_t v)
{
    switch (mode)
    {
    case 1: case 2: case 3: return dmax - d;
    case 4: case 5:
    {
        const uint64_t r = 2 * d / (avg ? avg : 1);
        const uint32_t group = r ? min(7u, 64u - (uint32_t)__clzll((long long)r)) : 0u;
        return 7u - group;
    }
    case 6: case 7: return d > avg ? dmax - d : dmax + 1;
    case 8: case 9: return d > avg ? 0u : 1u;
    case 10:
    {
        uint64_t z = seed ^ v;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return (z ^ (z >> 31)) & 0xffffffffull;
    }
    default: return 0;
    }
}

__global__ void k_relabel_keys(const uint32_t *__restrict__ dout, const uint32_t *__restrict__ din, uint32_t V,
                               uint32_t mode, uint64_t dmax, uint64_t avg, uint64_t seed, int b, uint64_t *keys)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
        keys[v] = (relabel_key(mode, mode_degree(mode, dout, din, v), dmax, avg, seed, v) << b) | v;
}

__global__ void k_labels_from_order(const uint64_t *__restrict__ keys, uint32_t V, uint64_t mask, uint32_t *label)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < V; i += gridDim.x * blockDim.x)
        label[keys[i] & mask] = i;
}

/* checks label is a permutation of 0..V-1 (every new id hit once) */
__global__ void k_perm_hits(const uint32_t *__restrict__ label, uint32_t V, uint32_t *hits, uint32_t *bad)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
    {
        const uint32_t l = label[v];
        if (l >= V || atomicAdd(hits + l, 1u) != 0u) atomicOr(bad, 1u);
    }
}

/* out may be ids (in place: each slot is read, then written, by one thread) */
__global__ void k_apply_labels(const uint32_t *ids, uint64_t n, const uint32_t *__restrict__ label, uint32_t *out)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = label[ids[i]];
}

int bits_for64(uint64_t x)
{
    int b = 0;
    while (b < 64 && (x >> b)) b++;
    return b;
}

/* a device scratch allocation freed at scope exit */
struct Scratch
{
    gg_graph *g;
    void *p = nullptr;
    size_t bytes = 0;
    Scratch(gg_graph *g_) : g(g_) {}
    gg_status alloc(size_t n)
    {
        bytes = n;
        return gg_dev_alloc(g, &p, n);
    }
    ~Scratch() { gg_dev_free(g, p, bytes); }
};

} // namespace

/* label[orig] = new for `mode` (1..10; 0 = identity) over device edge ids */
gg_status gg_relabel_device(gg_graph *g, uint32_t V, uint64_t E, const uint32_t *src, const uint32_t *dst,
                            uint32_t mode, uint64_t seed, uint32_t *label, cudaStream_t s)
{
    GgRange range("gg_relabel");
    if (mode > 10) return gg_fail(GG_ERR_INVALID, "relabelling mode must be 0..10 (11 takes labels from the caller)");
    Scratch degs(g), keys(g), tmp(g), counts(g), sums(g), flag(g);
    GG_CHECK(degs.alloc((size_t)V * 8 + 64));
    GG_CHECK(flag.alloc(64));
    uint32_t *dout = (uint32_t *)degs.p, *din = dout + V;
    GG_CUDA(cudaMemsetAsync(degs.p, 0, (size_t)V * 8 + 64, s));
    GG_CUDA(cudaMemsetAsync(flag.p, 0, 64, s));
    uint32_t *bad = (uint32_t *)flag.p;
    unsigned long long *dmax_d = (unsigned long long *)((char *)flag.p + 8);
    k_degree_count<<<grid_for(E, 256), 256, 0, s>>>(src, E, V, dout, bad);
    k_degree_count<<<grid_for(E, 256), 256, 0, s>>>(dst, E, V, din, bad);
    k_degree_max<<<grid_for(V, 256), 256, 0, s>>>(dout, din, V, mode, dmax_d);
    GG_CUDA(cudaGetLastError());
    unsigned long long hf[2] = {0, 0};
    GG_CHECK(gg_wait(s)); /* bounded, before a copy to pageable memory */
    GG_CUDA(cudaMemcpyAsync(hf, flag.p, 16, cudaMemcpyDeviceToHost, s));
    GG_CHECK(gg_wait(s));
    if (hf[0] & 0xffffffffull) return gg_fail(GG_ERR_INVALID, "edge list has a vertex id >= num_vertices");
    const uint64_t dmax = hf[1], avg = V ? E / V : 0;
    const int b = bits_for(V);
    int hi_bits = 0;
    switch (mode)
    {
    case 0: hi_bits = 0; break;
    case 1: case 2: case 3: hi_bits = bits_for64(dmax); break;
    case 4: case 5: hi_bits = 3; break;
    case 6: case 7: hi_bits = bits_for64(dmax + 1); break;
    case 8: case 9: hi_bits = 1; break;
    default: hi_bits = 32; break;
    }
    if (hi_bits + b > 64) return gg_fail(GG_ERR_INVALID, "degrees and ids do not fit one 64-bit sort key");
    GG_CHECK(keys.alloc((size_t)V * 8 + 16));
    GG_CHECK(tmp.alloc((size_t)V * 8 + 16));
    const uint32_t ntiles = (uint32_t)(((uint64_t)V + RDX_TILE - 1) / RDX_TILE);
    GG_CHECK(counts.alloc((size_t)RDX_BINS * (ntiles ? ntiles : 1) * 4));
    GG_CHECK(sums.alloc(((ntiles + COL_TILES - 1) / COL_TILES + 1) * RDX_BINS * 4));
    k_relabel_keys<<<grid_for(V, 256), 256, 0, s>>>(dout, din, V, mode, dmax, avg, seed, b, (uint64_t *)keys.p);
    GG_CUDA(cudaGetLastError());
    SortBufs B{(uint64_t *)keys.p, (uint64_t *)tmp.p, nullptr, nullptr, (uint32_t *)counts.p, (uint32_t *)sums.p};
    /* the words start in id order, so a stable sort of the key bits alone
     * leaves equal keys in id order */
    GG_CHECK(radix_sort(B, V, hi_bits + b, s, b));
    k_labels_from_order<<<grid_for(V, 256), 256, 0, s>>>(B.keys, V, (1ull << b) - 1ull, label);
    GG_CUDA(cudaGetLastError());
    return gg_wait(s);
}

gg_status gg_check_permutation(gg_graph *g, const uint32_t *label, uint32_t V, cudaStream_t s)
{
    Scratch hits(g), flag(g);
    GG_CHECK(hits.alloc((size_t)V * 4 + 16));
    GG_CHECK(flag.alloc(16));
    GG_CUDA(cudaMemsetAsync(hits.p, 0, (size_t)V * 4 + 16, s));
    GG_CUDA(cudaMemsetAsync(flag.p, 0, 16, s));
    k_perm_hits<<<grid_for(V, 256), 256, 0, s>>>(label, V, (uint32_t *)hits.p, (uint32_t *)flag.p);
    GG_CUDA(cudaGetLastError());
    uint32_t bad = 0;
    GG_CHECK(gg_wait(s)); /* bounded, before a copy to pageable memory */
    GG_CUDA(cudaMemcpyAsync(&bad, flag.p, 4, cudaMemcpyDeviceToHost, s));
    GG_CHECK(gg_wait(s));
    if (bad) return gg_fail(GG_ERR_INVALID, "label array is not a permutation of 0..V-1");
    return GG_OK;
}

gg_status gg_apply_labels(const uint32_t *ids, uint64_t n, const uint32_t *label, uint32_t *out, cudaStream_t s)
{
    k_apply_labels<<<grid_for(n, 256), 256, 0, s>>>(ids, n, label, out);
    GG_CUDA(cudaGetLastError());
    return GG_OK;
}
