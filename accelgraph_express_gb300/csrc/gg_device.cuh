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

__device__ __forceinline__ void atomic_add_acc(float *p, float v) { atomicAdd(p, v); }
__device__ __forceinline__ void atomic_add_acc(unsigned long long *p, unsigned long long v) { atomicAdd(p, v); }
__device__ __forceinline__ float atomic_take(float *p) { return atomicExch(p, 0.0f); }
__device__ __forceinline__ unsigned long long atomic_take(unsigned long long *p) { return atomicExch(p, 0ull); }

/* ---- merge-path tiles ------------------------------------------------------
 *
 * A CSR with V rows and E edges is the merge of two lists: the V row-end
 * offsets and the E edge slots.  Cutting that merge into tiles of
 * TILE_ITEMS items balances work whatever the degree distribution
 * (Merrill & Garland, "Merge-based parallel sparse matrix-vector
 * multiplication", SC'16).  coord[t] = (rows ended, edges consumed) at
 * diagonal t*TILE_ITEMS.
 *
 * A row whose items fall in more than one tile is finished by the last tile
 * to arrive: every participating tile adds its partial into acc[first tile
 * of the row] and bumps cnt[first tile]; the tile that brings the count to
 * the number of participants takes the total (resetting both) and runs the
 * row epilogue.  No tile waits for another.
 */

__device__ __forceinline__ uint2 merge_path_search(uint64_t diag, const uint32_t *row_end, uint32_t nrows,
                                                   uint32_t nedges, uint32_t edge_base)
{
    /* row_end[i] is the (absolute) end offset of row i; edges are numbered
     * from edge_base.  Returns (rows consumed, edges consumed). */
    uint64_t lo = diag > nedges ? diag - nedges : 0;
    uint64_t hi = diag < nrows ? diag : nrows;
    while (lo < hi)
    {
        uint64_t mid = (lo + hi) >> 1;
        if ((uint64_t)(row_end[mid] - edge_base) + mid < diag)
            lo = mid + 1;
        else
            hi = mid;
    }
    return make_uint2((uint32_t)lo, (uint32_t)(diag - lo));
}

/*
 * The tile engine.  Op supplies:
 *   typedef Acc;                             float or unsigned long long
 *   bool skip() const;                       whole launch is a no-op
 *   void load4(uint32_t e4, uint4 idx, Acc v[4]) const;
 *                                            values of edges e4..e4+3 with
 *                                            neighbour ids idx (pull gather)
 *   void finish(uint32_t row, Acc sum, double &err, uint32_t &act);
 *                                            row epilogue
 *   void block_end();                        called by every thread after
 *                                            the epilogue (block reductions)
 *   void reduce(double err, uint32_t act);   block totals (thread 0)
 */
template <int NT, int IPT, class Op>
__device__ __forceinline__ void tile_pull(const uint32_t *__restrict__ off, const uint32_t *__restrict__ adj,
                                          uint32_t V, const uint2 *__restrict__ coord,
                                          typename Op::Acc *g_acc, uint32_t *g_cnt, Op &op, uint32_t tile)
{
    typedef typename Op::Acc Acc;
    constexpr int TI = NT * IPT;
    __shared__ uint32_t s_off[TI + 2];
    __shared__ Acc s_val[TI];
    __shared__ Acc s_row[TI + 1];

    const uint2 c0 = coord[tile], c1 = coord[tile + 1];
    const uint32_t i0 = c0.x, j0 = c0.y, i1 = c1.x, j1 = c1.y;
    /* rows touched: i0 .. last_row; row i1 (if < V) may have edges here but
     * its end item lies in a later tile */
    const uint32_t last_row = i1 < V ? i1 : V - 1;
    const uint32_t nrows = (i1 < V || i0 < V) ? last_row - i0 + 1 : 0;
    const uint32_t nedges = j1 - j0;
    const uint32_t nitems = (i1 - i0) + nedges;

    /* s_off[k] = off[i0 + k], k = 0 .. nrows (start of each touched row and
     * the end of the last one) */
    for (uint32_t k = threadIdx.x; k <= nrows; k += NT)
        s_off[k] = off[i0 + k];
    for (uint32_t k = threadIdx.x; k < nrows + 1; k += NT)
        s_row[k] = Acc(0);

    /* gather: coalesced 16-byte index loads, independent value loads */
    {
        const uint32_t e_begin = j0 & ~3u;
        for (uint32_t e4 = e_begin + 4u * threadIdx.x; e4 < j1; e4 += 4u * NT)
        {
            const uint4 q = *reinterpret_cast<const uint4 *>(adj + e4);
            Acc v[4];
            op.load4(e4, q, v);
#pragma unroll
            for (int c = 0; c < 4; c++)
            {
                uint32_t e = e4 + c;
                if (e >= j0 && e < j1) s_val[e - j0] = v[c];
            }
        }
    }
    __syncthreads();

    /* merge-path consumption: IPT items per thread */
    {
        const uint32_t d = threadIdx.x * IPT;
        if (d < nitems)
        {
            /* rows of this tile whose end item is in this tile: i0 .. i1-1,
             * their ends are s_off[1 .. i1-i0] */
            uint2 p = merge_path_search(d, s_off + 1, i1 - i0, nedges, j0);
            uint32_t ri = p.x, ej = p.y;
            Acc sum = Acc(0);
            bool has = false;
            const uint32_t dend = min(d + IPT, nitems);
            for (uint32_t k = d; k < dend; k++)
            {
                /* end of local row ri relative to j0; the partial last row
                 * (ri == i1 - i0) never ends inside the tile */
                uint32_t rend = ri < i1 - i0 ? s_off[ri + 1] - j0 : 0xffffffffu;
                if (ej < rend)
                {
                    sum += s_val[ej];
                    ej++;
                    has = true;
                }
                else
                {
                    if (has) atomicAdd(&s_row[ri], sum);
                    sum = Acc(0);
                    has = false;
                    ri++;
                }
            }
            if (has) atomicAdd(&s_row[ri], sum);
        }
    }
    __syncthreads();

    /* row epilogue */
    double err = 0.0;
    uint32_t act = 0;
    const uint64_t tlo = (uint64_t)tile * TI, thi = tlo + TI;
    for (uint32_t k = threadIdx.x; k < nrows; k += NT)
    {
        const uint32_t r = i0 + k;
        const uint64_t first = (uint64_t)r + s_off[k];
        const uint64_t last = (uint64_t)r + s_off[k + 1]; /* the row's end item */
        const uint32_t t_first = (uint32_t)(first / TI), t_last = (uint32_t)(last / TI);
        if (t_first == t_last)
        {
            op.finish(r, s_row[k], err, act);
        }
        else
        {
            /* the row spans tiles: take part only if this tile holds some of
             * its items */
            const uint64_t a = first > tlo ? first : tlo;
            const uint64_t b = (last + 1) < thi ? (last + 1) : thi;
            if (a < b)
            {
                atomic_add_acc(&g_acc[t_first], s_row[k]);
                __threadfence();
                uint32_t prev = atomicAdd(&g_cnt[t_first], 1u);
                if (prev == t_last - t_first)
                {
                    __threadfence();
                    Acc total = atomic_take(&g_acc[t_first]);
                    g_cnt[t_first] = 0u;
                    op.finish(r, total, err, act);
                }
            }
        }
    }
    op.block_end();
    block_sum2<NT>(err, act);
    if (threadIdx.x == 0) op.reduce(err, act);
}

/*
 * Push counterpart: the same tiles over the out-CSR; every edge (row -> dst)
 * applies op.scatter(row, e, dst).  Per-row data is fetched once per thread
 * segment through op.row_value(row).
 */
template <int NT, int IPT, class Op>
__device__ __forceinline__ void tile_push(const uint32_t *__restrict__ off, const uint32_t *__restrict__ adj,
                                          uint32_t V, const uint2 *__restrict__ coord, Op &op, uint32_t tile)
{
    constexpr int TI = NT * IPT;
    __shared__ uint32_t s_off[TI + 2];
    __shared__ uint32_t s_adj[TI];

    const uint2 c0 = coord[tile], c1 = coord[tile + 1];
    const uint32_t i0 = c0.x, j0 = c0.y, i1 = c1.x, j1 = c1.y;
    const uint32_t last_row = i1 < V ? i1 : V - 1;
    const uint32_t nrows = (i1 < V || i0 < V) ? last_row - i0 + 1 : 0;
    const uint32_t nedges = j1 - j0;
    const uint32_t nitems = (i1 - i0) + nedges;

    for (uint32_t k = threadIdx.x; k <= nrows; k += NT)
        s_off[k] = off[i0 + k];
    {
        const uint32_t e_begin = j0 & ~3u;
        for (uint32_t e4 = e_begin + 4u * threadIdx.x; e4 < j1; e4 += 4u * NT)
        {
            const uint4 q = *reinterpret_cast<const uint4 *>(adj + e4);
            const uint32_t qa[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
            for (int c = 0; c < 4; c++)
            {
                uint32_t e = e4 + c;
                if (e >= j0 && e < j1) s_adj[e - j0] = qa[c];
            }
        }
    }
    __syncthreads();

    const uint32_t d = threadIdx.x * IPT;
    if (d < nitems)
    {
        uint2 p = merge_path_search(d, s_off + 1, i1 - i0, nedges, j0);
        uint32_t ri = p.x, ej = p.y;
        const uint32_t dend = min(d + IPT, nitems);
        bool have = false;
        typename Op::RowVal rv{};
        for (uint32_t k = d; k < dend; k++)
        {
            uint32_t rend = ri < i1 - i0 ? s_off[ri + 1] - j0 : 0xffffffffu;
            if (ej < rend)
            {
                if (!have) { rv = op.row_value(i0 + ri); have = true; }
                op.scatter(rv, j0 + ej, s_adj[ej]);
                ej++;
            }
            else
            {
                ri++;
                have = false;
            }
        }
    }
}

} // namespace gg
