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

/* Clear a sum slot that was just read.  The store is made to wait for the
 * load (a branch on the value read): on GB300 a store issued to a sector
 * whose L2 read miss is still outstanding stalls that sector, and a pass
 * that read and cleared 64 MB with an independent store ran 7x slower than
 * with this dependent one.  Slots already zero are left alone (-0.0 stays;
 * the atomics that later add into it give the same sums). */
__device__ __forceinline__ void clear_after_read(float *p, float seen)
{
    if (seen != 0.0f) *p = 0.0f;
}
__device__ __forceinline__ void clear_after_read(unsigned long long *p, unsigned long long seen)
{
    if (seen != 0ull) *p = 0ull;
}

/* ---- reductions --------------------------------------------------------- */

template <class T> __device__ __forceinline__ T warp_sum(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

/* Programmatic dependent launch: a kernel launched with
 * cudaLaunchAttributeProgrammaticStreamSerialization (gg_launch_pdl) may be
 * launched while the kernel before it on the stream still runs; it calls
 * pdl_wait before its first access to memory that kernel writes, which
 * returns once that kernel has completed and its writes are visible (at
 * once for a kernel launched without the attribute).  pdl_trigger lets the
 * next such kernel launch before this one has ended. */
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

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
 * A row whose items fall in more than one tile gets each tile's partial
 * sum added atomically; a row lying wholly in one tile is stored by that
 * tile.  No tile waits for another.
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

/* Gather loads issued where they are written (inline PTX is not moved), so a
 * tile's loads stay in flight while the previous tile is reduced; the
 * values are read-only for the launch (non-coherent path). */
__device__ __forceinline__ float ldg_val(const float *p)
{
    float v;
    asm volatile("ld.global.nc.f32 %0, [%1];" : "=f"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ uint32_t ldg_val(const uint32_t *p)
{
    uint32_t v;
    asm volatile("ld.global.nc.u32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ unsigned long long ldg_val(const unsigned long long *p)
{
    unsigned long long v;
    asm volatile("ld.global.nc.u64 %0, [%1];" : "=l"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ uint16_t ldg_val(const uint16_t *p)
{
    uint16_t v;
    asm volatile("ld.global.nc.u16 %0, [%1];" : "=h"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ uint8_t ldg_val(const uint8_t *p)
{
    uint32_t v;
    asm volatile("ld.global.nc.u8 %0, [%1];" : "=r"(v) : "l"(p));
    return (uint8_t)v;
}
__device__ __forceinline__ __nv_bfloat16 ldg_val(const __nv_bfloat16 *p)
{
    return __ushort_as_bfloat16(ldg_val(reinterpret_cast<const uint16_t *>(p)));
}
__device__ __forceinline__ __half ldg_val(const __half *p) { return __ushort_as_half(ldg_val(reinterpret_cast<const uint16_t *>(p))); }

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
/* wait until at most one committed group of this thread is still pending */
__device__ __forceinline__ void cp_async_wait_one() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

template <int IPT>
__device__ __forceinline__ void load_ids(uint32_t (&id)[IPT], const uint32_t *adj, uint32_t j0, uint32_t j1,
                                         uint32_t lane)
{
#pragma unroll
    for (int g = 0; g < IPT; g++)
    {
        const uint32_t e = j0 + lane + 32u * g;
        if (e < j1) id[g] = ldg_stream(adj + e);
    }
}

/* rows of a tile with at least one item in it: i0 .. last row (row i1 when
 * i1 < V has items here but ends in a later tile) */
__device__ __forceinline__ uint32_t tile_rows(uint2 c0, uint2 c1, uint32_t V)
{
    const uint32_t last_row = c1.x < V ? c1.x : V - 1;
    return (c1.x < V || c0.x < V) ? last_row - c0.x + 1 : 0;
}

/*
 * The pull engine: sums[r] = sum over the CSC row r of op's edge terms, for
 * every row, by persistent warps over merge-path tiles.  Op supplies:
 *   typedef Acc;                       float or unsigned long long
 *   typedef Raw;                       what one edge's gather loads
 *   Raw load(uint32_t e, uint32_t u) const;
 *                                      issue the loads of edge e with
 *                                      neighbour u (ldg_val)
 *   Acc value(const Raw &r) const;     the edge term, computed where the
 *                                      loads are first used
 * sums must be zero on entry for rows whose items span tiles: a row lying in
 * one tile is stored, the partials of a spanning row are added atomically
 * (the row epilogues that read sums clear it again).
 *
 * Each warp runs its tiles as a software pipeline: while tile A is reduced,
 * tile B's gathers and tile C's neighbour ids are in flight and tile B's row
 * offsets are landing in shared memory (cp.async, double-buffered), so a
 * tile's dependent load chain (ids, then values) overlaps the reduction of
 * the tile before it.  A tile is reduced along the merge path
 * (GG_TILE_IPT items per lane): a row ended inside a lane is stored
 * directly; the partial sum of the row open at the end of each lane is
 * combined across lanes by a warp-shuffle segmented scan.  Only __syncwarp
 * orders the phases.
 */
/* Per-warp shared staging of the pull engine: two buffers of row offsets
 * (each holding up to 3 words before the tile's first row, see stage_words,
 * 16-byte aligned), the tile's values and its row sums. */
template <int IPT, class Acc>
struct PullStage
{
    static constexpr uint32_t TW = 32 * IPT;
    static constexpr uint32_t OFFW = TW + 8;
    static constexpr size_t OFF_BYTES = (size_t)2 * OFFW * 4;
    static constexpr size_t VAL_BYTES = ((size_t)TW * sizeof(Acc) + 15) / 16 * 16;
    static constexpr size_t ROW_BYTES = ((size_t)(TW + 1) * sizeof(Acc) + 15) / 16 * 16;
    static constexpr size_t BYTES = OFF_BYTES + VAL_BYTES + ROW_BYTES;
};

/* The engine proper: this warp's tiles are tile, tile + nw, ...; s_offs
 * (2 * OFFW words), s_val (TW) and s_row (TW + 1) are its staging. */
template <int IPT, class Op>
__device__ __forceinline__ void warp_pull_sums_core(uint32_t *s_offs, typename Op::Acc *s_val,
                                                    typename Op::Acc *s_row, uint32_t tile, uint32_t nw,
                                                    const uint32_t *__restrict__ off, const uint32_t *__restrict__ adj,
                                                    uint32_t V, const uint2 *__restrict__ coord, uint32_t ntiles,
                                                    typename Op::Acc *sums, const Op &op)
{
    typedef typename Op::Acc Acc;
    typedef typename Op::Raw Raw;
    constexpr uint32_t TW = PullStage<IPT, Acc>::TW;
    constexpr uint32_t OFFW = PullStage<IPT, Acc>::OFFW;
    const uint32_t lane = threadIdx.x & 31;
    if (tile >= ntiles) return;

    /* pipeline state: A = tile (gathers in flight in val, offsets staged in
     * buffer buf), B = tile + nw (ids in flight in id, offsets staged in
     * buf ^ 1), C = tile + 2nw (coordinates only) */
    const uint2 zero2 = make_uint2(0, 0);
    uint2 a0 = coord[tile], a1 = coord[tile + 1];
    uint2 b0 = zero2, b1 = zero2, c0 = zero2, c1 = zero2;
    if (tile + nw < ntiles) { b0 = coord[tile + nw]; b1 = coord[tile + nw + 1]; }
    if (tile + 2 * nw < ntiles) { c0 = coord[tile + 2 * nw]; c1 = coord[tile + 2 * nw + 1]; }
    uint32_t id[IPT];
    Raw val[IPT];
    load_ids<IPT>(id, adj, a0.y, a1.y, lane);
    uint32_t buf = 0;
    uint32_t shA = stage_words(s_offs, off, a0.x, tile_rows(a0, a1, V) + 1, lane);
    cp_async_commit();
    uint32_t shB = 0;
    if (tile + nw < ntiles) shB = stage_words((s_offs + OFFW), off, b0.x, tile_rows(b0, b1, V) + 1, lane);
    cp_async_commit();
#pragma unroll
    for (int g = 0; g < IPT; g++)
    {
        const uint32_t e = a0.y + lane + 32u * g;
        if (e < a1.y) val[g] = op.load(e, id[g]);
    }
    if (tile + nw < ntiles) load_ids<IPT>(id, adj, b0.y, b1.y, lane);

    for (; tile < ntiles; tile += nw)
    {
        const bool hasB = tile + nw < ntiles, hasC = tile + 2 * nw < ntiles;
        /* B's gathers, C's ids, D's coordinates */
        Raw nv[IPT];
        if (hasB)
        {
#pragma unroll
            for (int g = 0; g < IPT; g++)
            {
                const uint32_t e = b0.y + lane + 32u * g;
                if (e < b1.y) nv[g] = op.load(e, id[g]);
            }
        }
        if (hasC) load_ids<IPT>(id, adj, c0.y, c1.y, lane);
        uint2 d0 = zero2, d1 = zero2;
        if (tile + 3 * nw < ntiles)
        {
            d0 = coord[tile + 3 * nw];
            d1 = coord[tile + 3 * nw + 1];
        }

        /* tile A */
        const uint32_t i0 = a0.x, j0 = a0.y, i1 = a1.x, j1 = a1.y;
        const uint32_t nedges = j1 - j0;
        const uint32_t nend = i1 - i0; /* local rows whose end item is in this tile */
        const uint32_t nitems = nend + nedges;
#pragma unroll
        for (int g = 0; g < IPT; g++)
        {
            const uint32_t e = j0 + lane + 32u * g;
            if (e < j1) s_val[e - j0] = op.value(val[g]);
        }
        cp_async_wait_one();
        __syncwarp();
        const uint32_t *s_off = (s_offs + buf * OFFW) + shA;

        /* merge-path consumption; the first row a lane ends may have begun
         * in earlier lanes, so its sum waits for the carry scan */
        const uint32_t d = lane * IPT;
        uint32_t first_row = 0xffffffffu, key = 0xffffffffu;
        Acc first_sum = Acc(0), carry = Acc(0);
        bool first_done = false;
        if (d < nitems)
        {
            uint2 p = merge_path_search(d, s_off + 1, nend, nedges, j0);
            uint32_t ri = p.x, ej = p.y;
            first_row = ri;
            uint32_t rend = ri < nend ? s_off[ri + 1] - j0 : 0xffffffffu;
            Acc sum = Acc(0);
            const uint32_t dend = min(d + IPT, nitems);
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
                    rend = ri < nend ? s_off[ri + 1] - j0 : 0xffffffffu;
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
            if (i1 < V)
            {
                const uint32_t m = __ballot_sync(0xffffffffu, key == nend);
                const Acc tot = m ? __shfl_sync(0xffffffffu, carry, 31 - __clz((int)m)) : Acc(0);
                if (lane == 0) s_row[nend] = tot;
            }
        }
        __syncwarp();

        /* rows ending here are stored, except row i0 when it began in an
         * earlier tile (off[i0] < j0); that one and the open row i1 add
         * their partials to sums */
        for (uint32_t k = lane; k < nend; k += 32)
        {
            if (k == 0 && s_off[0] < j0)
            {
                if (s_off[1] > j0) atomic_add_acc(&sums[i0], s_row[0]);
            }
            else
                sums[i0 + k] = s_row[k];
        }
        if (lane == 0 && i1 < V && s_off[nend] < j1) atomic_add_acc(&sums[i1], s_row[nend]);
        __syncwarp();

        /* C's offsets into A's buffer; rotate */
        uint32_t shC = 0;
        if (hasC) shC = stage_words((s_offs + buf * OFFW), off, c0.x, tile_rows(c0, c1, V) + 1, lane);
        cp_async_commit();
#pragma unroll
        for (int g = 0; g < IPT; g++) val[g] = nv[g];
        a0 = b0; a1 = b1; b0 = c0; b1 = c1; c0 = d0; c1 = d1;
        shA = shB; shB = shC;
        buf ^= 1u;
    }
    cp_async_wait_all();
}

/* the engine with static per-warp staging, WARPS warps per CTA */
template <int IPT, int WARPS, class Op>
__device__ __forceinline__ void warp_pull_sums(const uint32_t *__restrict__ off, const uint32_t *__restrict__ adj,
                                               uint32_t V, const uint2 *__restrict__ coord, uint32_t ntiles,
                                               typename Op::Acc *sums, const Op &op)
{
    typedef typename Op::Acc Acc;
    constexpr uint32_t TW = PullStage<IPT, Acc>::TW, OFFW = PullStage<IPT, Acc>::OFFW;
    __shared__ __align__(16) uint32_t sm_off[WARPS][2 * OFFW];
    __shared__ Acc sm_val[WARPS][TW];
    __shared__ Acc sm_row[WARPS][TW + 1];
    const uint32_t w = threadIdx.x >> 5;
    warp_pull_sums_core<IPT>(sm_off[w], sm_val[w], sm_row[w], blockIdx.x * WARPS + w, gridDim.x * WARPS, off, adj,
                             V, coord, ntiles, sums, op);
}

/* the engine with per-warp staging carved from dynamic shared memory at
 * `base` (blockDim.x / 32 warps of PullStage<IPT, Acc>::BYTES each) */
template <int IPT, class Op>
__device__ __forceinline__ void warp_pull_sums_dyn(unsigned char *base, const uint32_t *__restrict__ off,
                                                   const uint32_t *__restrict__ adj, uint32_t V,
                                                   const uint2 *__restrict__ coord, uint32_t ntiles,
                                                   typename Op::Acc *sums, const Op &op)
{
    typedef typename Op::Acc Acc;
    typedef PullStage<IPT, Acc> S;
    const uint32_t w = threadIdx.x >> 5, warps = blockDim.x >> 5;
    unsigned char *p = base + (size_t)w * S::BYTES;
    warp_pull_sums_core<IPT>(reinterpret_cast<uint32_t *>(p), reinterpret_cast<Acc *>(p + S::OFF_BYTES),
                             reinterpret_cast<Acc *>(p + S::OFF_BYTES + S::VAL_BYTES), blockIdx.x * warps + w,
                             gridDim.x * warps, off, adj, V, coord, ntiles, sums, op);
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

/*
 * Grid-wide barrier over the co-resident blocks of a cooperative launch, on
 * a control block `ctl` of GG_BAR_BYTES zeroed before the launch: the root
 * counter at 512, per group of blocks an arrival counter at 1024 + 128 g and
 * a release word at 4096 + 128 g (separate 128-byte lines, so the spinning
 * blocks of one group do not queue behind the arrivals or the other groups
 * at one L2 slice).  Two levels: blocks arrive at their group's counter, the
 * last of a group at the root, and the last at the root releases every
 * group.  The counters only grow (barrier `gen` completes a group at
 * (gen + 1) * group size arrivals and the root at (gen + 1) * groups), so
 * no arrival waits for a counter to be reset.  Ordering: each block's
 * writes are fenced before it arrives, the last arrivers fence before
 * passing on, and every block fences after it is released.  A wait gives up
 * after limit_ns (globaltimer) and sets *err; the block then reports false
 * and the caller leaves, so the other blocks give up at their next barrier
 * and the launch ends with *err set, the context intact.  Bytes 0..511 of
 * ctl are the caller's.
 */
constexpr unsigned int GG_BAR_GROUPS = 16;

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ bool grid_barrier(char *ctl, unsigned int *err, unsigned long long limit_ns,
                                             unsigned int &gen)
{
    __shared__ unsigned int s_ok;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        unsigned int *root = (unsigned int *)(ctl + 512);
        const unsigned int G = gridDim.x < GG_BAR_GROUPS ? gridDim.x : GG_BAR_GROUPS;
        const unsigned int grp = blockIdx.x % G;
        const unsigned int gsize = (gridDim.x - grp + G - 1) / G;
        unsigned int *count = (unsigned int *)(ctl + 1024 + 128 * grp);
        unsigned int *rel = (unsigned int *)(ctl + 4096 + 128 * grp);
        const unsigned int target = gen + 1;
        bool released = false, ok = true;
        __threadfence();
        if (atomicAdd(count, 1u) == target * gsize - 1)
        {
            __threadfence();
            if (atomicAdd(root, 1u) == target * G - 1)
            {
                __threadfence();
                for (unsigned int k = 0; k < G; k++) atomicExch((unsigned int *)(ctl + 4096 + 128 * k), target);
                released = true;
            }
        }
        if (!released)
        {
            const unsigned long long t0 = global_ns();
            while (*(volatile unsigned int *)rel != target)
            {
                if (global_ns() - t0 > limit_ns)
                {
                    atomicExch(err, 1u);
                    ok = false;
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
        s_ok = ok ? 1u : 0u;
    }
    __syncthreads();
    gen++;
    return s_ok != 0u;
}

} // namespace gg
