/*
 * Device-side helpers shared by the kernels: storage conversions, the
 * fixed-point formats, warp/block reductions, and the merge-path tile
 * engine that every pull gather and push scatter is built on.
 */
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cstdint>

#include "gg_internal.h"

namespace gg {

/* ---- storage types of gathered values ------------------------------------ */

template <class T> __device__ __forceinline__ float to_f32(T x);
template <> __device__ __forceinline__ float to_f32<float>(float x) { return x; }
template <> __device__ __forceinline__ float to_f32<__nv_bfloat16>(__nv_bfloat16 x) { return __bfloat162float(x); }
template <> __device__ __forceinline__ float to_f32<__half>(__half x) { return __half2float(x); }

template <class T> __device__ __forceinline__ T from_f32(float x);
template <> __device__ __forceinline__ float from_f32<float>(float x) { return x; }
template <> __device__ __forceinline__ __nv_bfloat16 from_f32<__nv_bfloat16>(float x) { return __float2bfloat16_rn(x); }
template <> __device__ __forceinline__ __half from_f32<__half>(float x) { return __float2half_rn(x); }

/* ---- fixed point (Q32.32 / Q16.16 / Q4.12 / Q2.6), same as the oracle ---- */

__device__ __forceinline__ uint64_t fx64_from_double(double x)
{
    double t = __dmul_rn(x, 4294967296.0);
    if (!(t > 0.0)) return 0ull;
    if (t >= 18446744073709551615.0) return ~0ull;
    return __double2ull_rz(t);
}
__device__ __forceinline__ double fx64_to_double(uint64_t f) { return __dmul_rn(__ull2double_rn(f), 1.0 / 4294967296.0); }
__device__ __forceinline__ uint64_t fx64_mul(uint64_t a, uint64_t b)
{
    /* (a*b) >> 32 of the 128-bit product */
    uint64_t lo = a * b;
    uint64_t hi = __umul64hi(a, b);
    return (hi << 32) | (lo >> 32);
}
__device__ __forceinline__ uint32_t fx_from_float(float x, double scale, uint32_t maxv)
{
    double t = __dmul_rn((double)x, scale);
    if (!(t > 0.0)) return 0u;
    if (t >= (double)maxv) return maxv;
    return __double2uint_rz(t);
}
__device__ __forceinline__ float fx_to_float(uint64_t f, double inv_scale)
{
    return __double2float_rn(__dmul_rn(__ull2double_rn(f), inv_scale));
}

/* ---- reductions --------------------------------------------------------- */

template <class T> __device__ __forceinline__ T warp_sum(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

/* Block-wide sum of (double, uint32) pairs; the result is valid in thread 0. */
template <int NT>
__device__ __forceinline__ void block_sum2(double &a, uint32_t &b)
{
    __shared__ double sa[NT / 32];
    __shared__ uint32_t sb[NT / 32];
    a = warp_sum(a);
    b = warp_sum(b);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) { sa[w] = a; sb[w] = b; }
    __syncthreads();
    if (w == 0)
    {
        a = l < NT / 32 ? sa[l] : 0.0;
        b = l < NT / 32 ? sb[l] : 0u;
        a = warp_sum(a);
        b = warp_sum(b);
    }
}

/* Asynchronous 4-byte global -> shared copy (cp.async, cached in L1): the
 * issuing thread holds no register for it and does not stall until
 * cp_async_wait_all.  Both addresses must be 4-byte aligned. */
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem)
{
    const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
/* Asynchronous 16-byte copy through L2 only (cp.async.cg), so staged
 * streams do not displace the L1-resident gather data.  Both addresses must
 * be 16-byte aligned. */
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
/* Wait for this thread's cp.async copies; a __syncwarp after it makes every
 * lane's copies visible to the whole warp. */
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

/* Streaming 4-byte load that does not allocate in L1 (the neighbour ids are
 * read once per launch). */
__device__ __forceinline__ uint32_t ldg_stream(const uint32_t *p)
{
    uint32_t v;
    asm volatile("ld.global.nc.L1::no_allocate.u32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}

/*
 * One warp copies src[i0 .. i0+n) into shared memory asynchronously, word
 * i0+k landing at dst[(i0 & 3) + k]; dst must be 16-byte aligned with room
 * for n + 3 words.  From a 16-byte-aligned src the body moves in 16-byte
 * chunks starting at the aligned word at or below i0 (words before i0 are
 * copied too, never words at or past i0+n); the last 1-3 words and any
 * unaligned src go word by word.  Returns i0 & 3.
 */
__device__ __forceinline__ uint32_t stage_words(uint32_t *dst, const uint32_t *src, uint32_t i0, uint32_t n,
                                                uint32_t lane)
{
    const uint32_t first = i0 & 3u;
    if ((reinterpret_cast<uintptr_t>(src) & 15u) == 0)
    {
        const uint32_t base = i0 - first, total = first + n, full = total >> 2;
        for (uint32_t c = lane; c < full; c += 32) cp_async16(dst + 4u * c, src + base + 4u * c);
        if (lane < (total & 3u)) cp_async4(dst + 4u * full + lane, src + base + 4u * full + lane);
    }
    else
        for (uint32_t k = lane; k < n; k += 32) cp_async4(dst + first + k, src + i0 + k);
    return first;
}

__device__ __forceinline__ void atomic_add_acc(float *p, float v) { atomicAdd(p, v); }
__device__ __forceinline__ void atomic_add_acc(unsigned long long *p, unsigned long long v) { atomicAdd(p, v); }
__device__ __forceinline__ float atomic_take(float *p) { return atomicExch(p, 0.0f); }
__device__ __forceinline__ unsigned long long atomic_take(unsigned long long *p) { return atomicExch(p, 0ull); }

/* ---- merge-path tiles ------------------------------------------------------
 *
 * A CSR with V rows and E edges is the merge of two lists: the V row-end
 * offsets and the E edge slots.  Cutting that merge into tiles of
 * GG_TILE_ITEMS items balances work whatever the degree distribution
 * (Merrill & Garland, "Merge-based parallel sparse matrix-vector
 * multiplication", SC'16).  coord[t] = (rows ended, edges consumed) at
 * diagonal t*GG_TILE_ITEMS.  Each tile is consumed by one warp.
 *
 * A row whose items fall in more than one tile is finished after the launch:
 * every participating tile adds its partial into acc[first tile of the row]
 * and warp_pull_fixup, a separate launch, runs the row epilogue on the
 * total.  No tile waits for another.  A row lying wholly in one tile is
 * finished by that tile alone (the tile before it also lists it, as its
 * partial last row, when it ends exactly at the row's first edge).
 */

__device__ __forceinline__ uint2 merge_path_search(uint32_t diag, const uint32_t *row_end, uint32_t nrows,
                                                   uint32_t nedges, uint32_t edge_base)
{
    /* row_end[i] is the (absolute) end offset of local row i; edges are
     * numbered from edge_base.  Returns (rows consumed, edges consumed). */
    uint32_t lo = diag > nedges ? diag - nedges : 0;
    uint32_t hi = diag < nrows ? diag : nrows;
    while (lo < hi)
    {
        uint32_t mid = (lo + hi) >> 1;
        if ((row_end[mid] - edge_base) + mid < diag)
            lo = mid + 1;
        else
            hi = mid;
    }
    return make_uint2(lo, diag - lo);
}

/* Per-warp tile geometry shared by the pull and push engines. */
struct TileGeom
{
    uint32_t i0, j0, i1, j1, nrows, nedges, nitems;
    __device__ __forceinline__ void load(const uint2 *coord, uint32_t tile, uint32_t V)
    {
        const uint2 c0 = coord[tile], c1 = coord[tile + 1];
        i0 = c0.x; j0 = c0.y; i1 = c1.x; j1 = c1.y;
        /* rows touched: i0 .. last_row; row i1 (if < V) may have edges here
         * but its end item lies in a later tile */
        const uint32_t last_row = i1 < V ? i1 : V - 1;
        nrows = (i1 < V || i0 < V) ? last_row - i0 + 1 : 0;
        nedges = j1 - j0;
        nitems = (i1 - i0) + nedges;
    }
};

/*
 * The pull engine (persistent warps).  Op supplies:
 *   typedef Acc;                        float or unsigned long long
 *   typedef RowPre;                     per-row data the epilogue needs
 *   Acc load1(uint32_t e, uint32_t u) const;
 *                                       value of edge e with neighbour u
 *                                       (the gather)
 *   RowPre prefetch(uint32_t row) const;
 *                                       per-row data, loaded directly
 *   static constexpr uint32_t PRE_WORDS;
 *   void stage(uint32_t i0, uint32_t n, uint32_t lane, uint32_t *s, uint32_t stride) const;
 *                                       the same data for rows i0..i0+n-1
 *                                       as PRE_WORDS planes of 32-bit words
 *                                       (plane p at s + p*stride), each
 *                                       copied with stage_words
 *   RowPre unstage(uint32_t row, const uint32_t *s, uint32_t j, uint32_t stride) const;
 *                                       row's data from index j of the planes
 *   void finish(uint32_t row, Acc sum, const RowPre &pre, double &err, uint32_t &act);
 *                                       row epilogue
 *   void warp_end(double err, uint32_t act);
 *                                       called by every lane at the end
 *                                       (warp reductions and atomics)
 * Per tile every load is issued up front, together: the neighbour ids (one
 * warp instruction covering 32 consecutive edges), the next tile's
 * coordinates, and, as asynchronous copies into shared memory, the tile's
 * row offsets and every row's epilogue data; then the neighbour values.  A
 * tile holds up to GG_TILE_ITEMS + 1 rows (R-MAT graphs have long runs of
 * in-degree-0 and -1 vertices), and the copies keep their loads from forming
 * one dependent round trip per 32 rows.  With the value gather saturating L2
 * sector requests, each extra dependent round trip per tile would cost a
 * full queueing latency.  The values are staged in shared memory and consumed
 * along the merge path (GG_TILE_IPT items per lane).  A row ended inside a
 * lane is stored directly; the partial sum of the row open at the end of
 * each lane is combined across lanes by a warp-shuffle segmented scan, so no
 * shared-memory atomics are needed.  Rows whose items span tiles add their
 * in-tile partial to acc[first tile of the row] with a fire-and-forget
 * reduction and are finished by warp_pull_fixup after the launch.  Only
 * __syncwarp orders the phases.
 */
template <int IPT, int WARPS, class Op>
__device__ __forceinline__ void warp_pull(const uint32_t *__restrict__ off, const uint32_t *__restrict__ adj,
                                          uint32_t V, const uint2 *__restrict__ coord, uint32_t ntiles,
                                          typename Op::Acc *g_acc, Op &op)
{
    typedef typename Op::Acc Acc;
    constexpr uint32_t TW = 32 * IPT;
    /* staged planes hold up to 3 words before the tile's first row
     * (stage_words) and stay 16-byte aligned; an Op without per-row data
     * keeps a token 4-word array */
    constexpr uint32_t OFFW = TW + 8, PREW = TW + 4;
    constexpr uint32_t PRE_ALL = Op::PRE_WORDS > 0 ? Op::PRE_WORDS * PREW : 4;
    __shared__ __align__(16) uint32_t sm_off[WARPS][OFFW];
    __shared__ __align__(16) uint32_t sm_pre[WARPS][PRE_ALL];
    __shared__ Acc sm_val[WARPS][TW];
    __shared__ Acc sm_row[WARPS][TW + 1];
    const uint32_t w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t *const s_offb = sm_off[w];
    Acc *s_val = sm_val[w];
    Acc *s_row = sm_row[w];
    uint32_t *const s_pre = sm_pre[w];
    double err = 0.0;
    uint32_t act = 0;
    const uint32_t nw = gridDim.x * WARPS;
    uint32_t tile = blockIdx.x * WARPS + w;
    uint2 c0 = make_uint2(0, 0), c1 = make_uint2(0, 0);
    if (tile < ntiles)
    {
        c0 = coord[tile];
        c1 = coord[tile + 1];
    }
    for (; tile < ntiles; tile += nw)
    {
        TileGeom t;
        t.i0 = c0.x; t.j0 = c0.y; t.i1 = c1.x; t.j1 = c1.y;
        {
            const uint32_t last_row = t.i1 < V ? t.i1 : V - 1;
            t.nrows = (t.i1 < V || t.i0 < V) ? last_row - t.i0 + 1 : 0;
            t.nedges = t.j1 - t.j0;
            t.nitems = (t.i1 - t.i0) + t.nedges;
        }
        /* every load of this tile in flight together (nedges <= TW,
         * nrows <= TW + 1) */
        uint32_t id[IPT];
#pragma unroll
        for (int g = 0; g < IPT; g++)
        {
            const uint32_t e = t.j0 + lane + 32u * g;
            if (e < t.j1) id[g] = ldg_stream(adj + e);
        }
        /* row i0+k of every staged plane sits at index shift+k */
        const uint32_t shift = stage_words(s_offb, off, t.i0, t.nrows + 1, lane);
        const uint32_t *s_off = s_offb + shift;
        if constexpr (Op::PRE_WORDS > 0) op.stage(t.i0, t.nrows, lane, s_pre, PREW);
        {
            const uint32_t nt = tile + nw;
            if (nt < ntiles)
            {
                c0 = coord[nt];
                c1 = coord[nt + 1];
            }
        }
#pragma unroll
        for (int g = 0; g < IPT; g++)
        {
            const uint32_t e = t.j0 + lane + 32u * g;
            if (e < t.j1) s_val[e - t.j0] = op.load1(e, id[g]);
        }
        cp_async_wait_all();
        __syncwarp();

        /* merge-path consumption; the first row a lane ends may have begun
         * in earlier lanes, so its sum waits for the carry scan */
        const uint32_t nend = t.i1 - t.i0; /* local rows whose end is in this tile */
        const uint32_t d = lane * IPT;
        uint32_t first_row = 0xffffffffu, key = 0xffffffffu;
        Acc first_sum = Acc(0), carry = Acc(0);
        bool first_done = false;
        if (d < t.nitems)
        {
            uint2 p = merge_path_search(d, s_off + 1, nend, t.nedges, t.j0);
            uint32_t ri = p.x, ej = p.y;
            first_row = ri;
            uint32_t rend = ri < nend ? s_off[ri + 1] - t.j0 : 0xffffffffu;
            Acc sum = Acc(0);
            const uint32_t dend = min(d + IPT, t.nitems);
            for (uint32_t k = d; k < dend; k++)
            {
                if (ej < rend)
                {
                    sum += s_val[ej];
                    ej++;
                }
                else
                {
                    if (!first_done)
                    {
                        first_sum = sum;
                        first_done = true;
                    }
                    else
                        s_row[ri] = sum;
                    sum = Acc(0);
                    ri++;
                    rend = ri < nend ? s_off[ri + 1] - t.j0 : 0xffffffffu;
                }
            }
            key = ri;
            carry = sum;
        }
        /* segmented inclusive scan of the open-row partials, keyed by row
         * (keys are non-decreasing across lanes) */
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const uint32_t k2 = __shfl_up_sync(0xffffffffu, key, o);
            const Acc v2 = __shfl_up_sync(0xffffffffu, carry, o);
            if (lane >= (uint32_t)o && k2 == key) carry += v2;
        }
        {
            const uint32_t kp = __shfl_up_sync(0xffffffffu, key, 1);
            const Acc vp = __shfl_up_sync(0xffffffffu, carry, 1);
            if (first_done) s_row[first_row] = first_sum + ((lane > 0 && kp == first_row) ? vp : Acc(0));
            /* the row left open at the end of the tile (row i1) */
            if (t.i1 < V)
            {
                const uint32_t m = __ballot_sync(0xffffffffu, key == nend);
                const Acc tot = m ? __shfl_sync(0xffffffffu, carry, 31 - __clz((int)m)) : Acc(0);
                if (lane == 0) s_row[nend] = tot;
            }
        }
        __syncwarp();

        /* row epilogue: rows wholly inside the tile are finished here; rows
         * spanning tiles send their partial to the fix-up pass */
        const uint64_t tlo = (uint64_t)tile * TW, thi = tlo + TW;
        for (uint32_t k = lane; k < t.nrows; k += 32)
        {
            const uint32_t r = t.i0 + k;
            const uint64_t first = (uint64_t)r + s_off[k];
            const uint64_t last = (uint64_t)r + s_off[k + 1]; /* the row's end item */
            const uint32_t t_first = (uint32_t)(first / TW), t_last = (uint32_t)(last / TW);
            if (t_first == t_last)
            {
                if (t_first == tile) op.finish(r, s_row[k], op.unstage(r, s_pre, shift + k, PREW), err, act);
            }
            else
            {
                const uint64_t a = first > tlo ? first : tlo;
                const uint64_t b = (last + 1) < thi ? (last + 1) : thi;
                if (a < b) atomic_add_acc(&g_acc[t_first], s_row[k]);
            }
        }
        __syncwarp();
    }
    op.warp_end(err, act);
}

/*
 * After warp_pull: finish every row whose items span tiles.  Such a row
 * starts in tile t and is left open at t's end, i.e. it is row coord[t+1].x
 * with at least one edge before coord[t+1].y and its first item inside t.
 * acc[t] holds the sum of all its tiles' partials (the launch boundary
 * orders them); it is reset for the next launch.  One thread per tile.
 */
template <class Op>
__device__ __forceinline__ void warp_pull_fixup(const uint32_t *__restrict__ off, uint32_t V,
                                                const uint2 *__restrict__ coord, uint32_t ntiles, uint32_t tw,
                                                typename Op::Acc *g_acc, Op &op)
{
    typedef typename Op::Acc Acc;
    double err = 0.0;
    uint32_t act = 0;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < ntiles; t += gridDim.x * blockDim.x)
    {
        const uint2 c1 = coord[t + 1];
        const uint32_t r = c1.x;
        if (r >= V) continue;
        const uint32_t o = off[r];
        if (o < c1.y && (uint64_t)r + o >= (uint64_t)t * tw)
        {
            const Acc total = g_acc[t];
            g_acc[t] = Acc(0);
            op.finish(r, total, op.prefetch(r), err, act);
        }
    }
    op.warp_end(err, act);
}

/*
 * The push engine: the same warp tiles over the out-CSR; every edge
 * (row -> dst) applies op.scatter(row value, edge, dst).  Per-row data is
 * fetched once per lane segment through op.row_value(row).
 */
template <int IPT, int WARPS, class Op>
__device__ __forceinline__ void warp_push(const uint32_t *__restrict__ off, const uint32_t *__restrict__ adj,
                                          uint32_t V, const uint2 *__restrict__ coord, uint32_t ntiles, Op &op)
{
    constexpr uint32_t TW = 32 * IPT;
    __shared__ __align__(16) uint32_t sm_off[WARPS][TW + 8];
    __shared__ __align__(16) uint32_t sm_adj[WARPS][TW + 4];
    const uint32_t w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t nw = gridDim.x * WARPS;
    for (uint32_t tile = blockIdx.x * WARPS + w; tile < ntiles; tile += nw)
    {
        TileGeom t;
        t.load(coord, tile, V);
        /* edge j0+i at s_adj[i], row i0+k's offset at s_off[k] */
        const uint32_t *s_adj = sm_adj[w] + stage_words(sm_adj[w], adj, t.j0, t.nedges, lane);
        const uint32_t *s_off = sm_off[w] + stage_words(sm_off[w], off, t.i0, t.nrows + 1, lane);
        cp_async_wait_all();
        __syncwarp();
        const uint32_t d = lane * IPT;
        if (d < t.nitems)
        {
            const uint32_t nend = t.i1 - t.i0;
            uint2 p = merge_path_search(d, s_off + 1, nend, t.nedges, t.j0);
            uint32_t ri = p.x, ej = p.y;
            const uint32_t *ids = s_adj;
            uint32_t rend = ri < nend ? s_off[ri + 1] - t.j0 : 0xffffffffu;
            const uint32_t dend = min(d + IPT, t.nitems);
            bool have = false;
            typename Op::RowVal rv{};
            for (uint32_t k = d; k < dend; k++)
            {
                if (ej < rend)
                {
                    if (!have) { rv = op.row_value(t.i0 + ri); have = true; }
                    op.scatter(rv, t.j0 + ej, ids[ej]);
                    ej++;
                }
                else
                {
                    ri++;
                    have = false;
                    rend = ri < nend ? s_off[ri + 1] - t.j0 : 0xffffffffu;
                }
            }
        }
        __syncwarp();
    }
}

/* warp sums of the per-lane residual terms, then one atomic per warp */
__device__ __forceinline__ void warp_reduce_to(double err, uint32_t act, double *err_dst, uint32_t *act_dst)
{
    err = warp_sum(err);
    act = warp_sum(act);
    if ((threadIdx.x & 31) == 0)
    {
        if (err != 0.0) atomicAdd(err_dst, err);
        if (act) atomicAdd(act_dst, act);
    }
}

__device__ __forceinline__ void warp_max_to(uint32_t v, uint32_t *dst)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_down_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0 && v) atomicMax(dst, v);
}

} // namespace gg
