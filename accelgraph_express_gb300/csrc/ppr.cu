/*
 * Batched personalised PageRank: K rank vectors over one graph, all advanced
 * by one pull gather per iteration.  There is no counterpart in the
 * reference's C API; per vector the arithmetic is the reference's pull
 * PageRank (pageRank.c:1026-1069: contribution = rank / outdeg, 0 for
 * outdeg 0, no dangling redistribution) with the uniform teleport replaced
 * by a teleport to the vector's seed set S_k:
 *     rank_0[v][k]  = c_k(v) / |S_k|              (c_k(v): occurrences of v in S_k)
 *     contrib[v][k] = rank[v][k] / outdeg(v)
 *     rank'[v][k]   = (1-d) c_k(v) / |S_k| + d * sum over in-edges (u,v) of contrib[u][k]
 *
 * Layout: contributions vertex-major, [V][KP] with KP = K rounded up to 16,
 * 32 or 64, stored in FP32 or BF16 and summed in FP32.  At KP = 64 BF16 one
 * vertex's contributions are one 128-byte line, so every edge of the CSC
 * gathers one full line.  A group of KP/4 lanes owns a merge-path tile and
 * walks it edge by edge, each lane summing four vectors from one 8-byte
 * (BF16) or 16-byte (FP32) load; several groups share a warp, and a batch of
 * edges' rows is in flight while the previous ones are summed.  Rows are
 * finished where they end: rank = teleport + d * sum (the teleport row comes
 * through a per-vertex seed index), contribution = rank * (1 / outdeg) with
 * the reciprocal computed once per vertex (within an ulp of the division:
 * the division, 4 per lane per row end, had made the row ends the bulk of
 * the work); FP32 ranks are only written by the last iteration.  A row
 * spanning tiles leaves its partial sum in per-tile slots (the tile where it began or that it crosses: `tail`;
 * the tile where it ends: `head`) and k_ppr_fixup adds them in tile order, so
 * every vector's result is deterministic and independent of the vectors
 * batched with it.
 */
#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "gg_device.cuh"

namespace {

using namespace gg;

constexpr uint32_t NO_SEED = 0xffffffffu;

/* VPL stored values per lane, read in one access of 4, 8 or 16 bytes */
template <class CT, int VPL> struct VecIO;
template <int VPL> struct Bf16IO
{
    static constexpr int W = VPL / 2; /* 32-bit words per lane */
    struct Raw
    {
        uint32_t w[W];
    };
    static __device__ __forceinline__ Raw load(const __nv_bfloat16 *p)
    {
        Raw r;
        if constexpr (W == 4)
            asm volatile("ld.global.nc.v4.u32 {%0, %1, %2, %3}, [%4];"
                         : "=r"(r.w[0]), "=r"(r.w[1]), "=r"(r.w[2]), "=r"(r.w[3]) : "l"(p));
        else if constexpr (W == 2)
            asm volatile("ld.global.nc.v2.u32 {%0, %1}, [%2];" : "=r"(r.w[0]), "=r"(r.w[1]) : "l"(p));
        else
            asm volatile("ld.global.nc.u32 %0, [%1];" : "=r"(r.w[0]) : "l"(p));
        return r;
    }
    /* through L2 only: contributions rewritten inside the persistent launch */
    static __device__ __forceinline__ Raw load_cg(const __nv_bfloat16 *p)
    {
        Raw r;
        if constexpr (W == 4)
            asm volatile("ld.global.cg.v4.u32 {%0, %1, %2, %3}, [%4];"
                         : "=r"(r.w[0]), "=r"(r.w[1]), "=r"(r.w[2]), "=r"(r.w[3]) : "l"(p));
        else if constexpr (W == 2)
            asm volatile("ld.global.cg.v2.u32 {%0, %1}, [%2];" : "=r"(r.w[0]), "=r"(r.w[1]) : "l"(p));
        else
            asm volatile("ld.global.cg.u32 %0, [%1];" : "=r"(r.w[0]) : "l"(p));
        return r;
    }
    /* element 2i is the low half of word i (little-endian); BF16 -> FP32 is exact */
    static __device__ __forceinline__ void add(float *acc, const Raw &r)
    {
#pragma unroll
        for (int i = 0; i < W; i++)
        {
            acc[2 * i] += __uint_as_float(r.w[i] << 16);
            acc[2 * i + 1] += __uint_as_float(r.w[i] & 0xffff0000u);
        }
    }
    static __device__ __forceinline__ void store(__nv_bfloat16 *p, const float *c)
    {
        uint32_t w[W];
#pragma unroll
        for (int i = 0; i < W; i++)
        {
            const __nv_bfloat162 h = __floats2bfloat162_rn(c[2 * i], c[2 * i + 1]);
            w[i] = *reinterpret_cast<const uint32_t *>(&h);
        }
        if constexpr (W == 4)
            *reinterpret_cast<uint4 *>(p) = make_uint4(w[0], w[1], w[2], w[3]);
        else if constexpr (W == 2)
            *reinterpret_cast<uint2 *>(p) = make_uint2(w[0], w[1]);
        else
            *reinterpret_cast<uint32_t *>(p) = w[0];
    }
};
template <int VPL> struct F32IO
{
    struct Raw
    {
        float v[VPL];
    };
    static __device__ __forceinline__ Raw load(const float *p)
    {
        Raw r;
        if constexpr (VPL == 4)
            asm volatile("ld.global.nc.v4.f32 {%0, %1, %2, %3}, [%4];"
                         : "=f"(r.v[0]), "=f"(r.v[1]), "=f"(r.v[2]), "=f"(r.v[3]) : "l"(p));
        else
            asm volatile("ld.global.nc.v2.f32 {%0, %1}, [%2];" : "=f"(r.v[0]), "=f"(r.v[1]) : "l"(p));
        return r;
    }
    static __device__ __forceinline__ Raw load_cg(const float *p)
    {
        Raw r;
        if constexpr (VPL == 4)
            asm volatile("ld.global.cg.v4.f32 {%0, %1, %2, %3}, [%4];"
                         : "=f"(r.v[0]), "=f"(r.v[1]), "=f"(r.v[2]), "=f"(r.v[3]) : "l"(p));
        else
            asm volatile("ld.global.cg.v2.f32 {%0, %1}, [%2];" : "=f"(r.v[0]), "=f"(r.v[1]) : "l"(p));
        return r;
    }
    static __device__ __forceinline__ void add(float *acc, const Raw &r)
    {
#pragma unroll
        for (int i = 0; i < VPL; i++) acc[i] += r.v[i];
    }
    static __device__ __forceinline__ void store(float *p, const float *c)
    {
        if constexpr (VPL == 4)
            *reinterpret_cast<float4 *>(p) = make_float4(c[0], c[1], c[2], c[3]);
        else
            *reinterpret_cast<float2 *>(p) = make_float2(c[0], c[1]);
    }
};
template <int V> struct VecIO<__nv_bfloat16, V> : Bf16IO<V>
{
    static constexpr int VPL = V;
};
template <int V> struct VecIO<float, V> : F32IO<V>
{
    static constexpr int VPL = V;
};

/* values per lane of the PPR gather and edges per batch (rows in flight
 * per lane group, at most one per lane of the group), by storage and row
 * width KP, as measured on R-MAT-22 (20 iterations, GTEPS, BF16 / FP32):
 *   KP = 64: 4 per lane (one 8- or 16-byte load), batches of 6 / 4:
 *            2,249 / 1,856 (2 per lane: 2,037 / 1,330; 8 BF16 per lane
 *            with batches of 4: 2,032, of 8: 1,510)
 *   KP = 32: BF16 2 per lane, batches of 8: 1,427 (4 per lane: 1,406);
 *            FP32 4 per lane, batches of 4: 1,281 (2 per lane: 1,253)
 *   KP = 16: 2 per lane, batches of 8: 908 / 782 (4 per lane: 712 / 671) */
template <class CT, int KP> constexpr int ppr_vpl()
{
    return (KP == 16 || (sizeof(CT) == 2 && KP == 32)) ? 2 : 4;
}
template <class CT, int KP> using PprIO = VecIO<CT, ppr_vpl<CT, KP>()>;

/* VPL consecutive floats (aligned to 4 * min(VPL, 4) bytes) */
template <int VPL>
__device__ __forceinline__ void load_f32(const float *p, float *v)
{
    if constexpr (VPL % 4 == 0)
    {
#pragma unroll
        for (int i = 0; i < VPL; i += 4)
        {
            const float4 t = *reinterpret_cast<const float4 *>(p + i);
            v[i] = t.x;
            v[i + 1] = t.y;
            v[i + 2] = t.z;
            v[i + 3] = t.w;
        }
    }
    else
    {
#pragma unroll
        for (int i = 0; i < VPL; i += 2)
        {
            const float2 t = *reinterpret_cast<const float2 *>(p + i);
            v[i] = t.x;
            v[i + 1] = t.y;
        }
    }
}
template <int VPL>
__device__ __forceinline__ void store_f32(float *p, const float *v)
{
    if constexpr (VPL % 4 == 0)
    {
#pragma unroll
        for (int i = 0; i < VPL; i += 4)
            *reinterpret_cast<float4 *>(p + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
    }
    else
    {
#pragma unroll
        for (int i = 0; i < VPL; i += 2) *reinterpret_cast<float2 *>(p + i) = make_float2(v[i], v[i + 1]);
    }
}

template <class CT>
struct PprArgs
{
    const uint32_t *off, *adj, *seed_idx;
    const float *inv_deg; /* 1 / out-degree, 0 for out-degree 0 */
    const uint2 *coord;
    uint32_t ntiles, V, E;
    uint32_t tile_log2; /* merge items per tile, a power of two (512 by default, the tuned size otherwise) */
    const CT *cin;
    CT *cout;
    float *rank;       /* [V][rs]: ranks of the vectors in rank_mask are written here */
    unsigned long long rank_mask; /* vectors whose ranks this iteration writes (their last) */
    unsigned long long zero_mask; /* vectors whose contributions are stored as zero (a freed slot) */
    const float *tele; /* [nseeds][rs]: (1-d) c_k(v) / |S_k| of seed vertex i */
    float *head;       /* [ntiles][KP]: partial of the row that ends in the tile but began before it */
    float *tail;       /* [ntiles][KP]: partial of the row left open at the tile's end */
    float damp;
};

/* what changes from one iteration to the next: the contributions read and
 * written, and the vectors whose ranks this iteration writes (kept apart
 * from PprArgs so that the persistent kernel reads PprArgs from its
 * parameter space instead of copying it into registers) */
template <class CT>
struct PprIter
{
    const CT *cin;
    CT *cout;
    unsigned long long rank_mask;
};

/* the stores of a row end in an iteration where some vectors write their
 * ranks or retire (rare: kept out of line so the unrolled edge loop, which
 * inlines the row end at every edge of a batch, stays small; inlined, it
 * cost the K = 64 gather 20% on R-MAT-22) */
template <int KP, class CT>
__device__ __noinline__ void ppr_store_masked(CT *cout, float *rank, unsigned long long rank_mask,
                                              unsigned long long zero_mask, size_t o, const float *r, float *c,
                                              uint32_t gl)
{
    constexpr int VPL = PprIO<CT, KP>::VPL;
    const uint32_t zero = (uint32_t)(zero_mask >> (VPL * gl)) & ((1u << VPL) - 1u);
    const uint32_t want = (uint32_t)(rank_mask >> (VPL * gl)) & ((1u << VPL) - 1u);
#pragma unroll
    for (int k = 0; k < VPL; k++)
        if (zero >> k & 1u) c[k] = 0.0f;
    PprIO<CT, KP>::store(cout + o, c);
    if (want == (1u << VPL) - 1u)
        store_f32<VPL>(rank + o, r);
    else
#pragma unroll
        for (int k = 0; k < VPL; k++)
            if (want >> k & 1u) rank[o + k] = r[k];
}

/* rank and contribution of row r from its sums (VPL vectors of this lane):
 * contribution = rank * (1 / out-degree), the reciprocal computed once per
 * vertex (within an ulp of rank / out-degree; 0 without out-edges).
 * RS: values per vertex row of cin / cout / rank / tele -- KP, or 64 when
 * only the first KP of wider rows are run (the server's continuous batch) */
template <int KP, int RS, class CT>
__device__ __forceinline__ void ppr_finish(const PprArgs<CT> &a, const PprIter<CT> &it, uint32_t r, const float *s,
                                           uint32_t si, float inv, uint32_t gl)
{
    constexpr int VPL = PprIO<CT, KP>::VPL;
    float rr[VPL], c[VPL];
#pragma unroll
    for (int k = 0; k < VPL; k++) rr[k] = __fmul_rn(a.damp, s[k]);
    if (si != NO_SEED)
    {
        float t[VPL];
        load_f32<VPL>(a.tele + (size_t)si * RS + VPL * gl, t);
#pragma unroll
        for (int k = 0; k < VPL; k++) rr[k] = __fadd_rn(t[k], rr[k]);
    }
#pragma unroll
    for (int k = 0; k < VPL; k++) c[k] = __fmul_rn(rr[k], inv);
    const size_t o = (size_t)r * RS + VPL * gl;
    if ((it.rank_mask | a.zero_mask) == 0ull)
        PprIO<CT, KP>::store(it.cout + o, c);
    else
        ppr_store_masked<KP, CT>(it.cout, a.rank, it.rank_mask, a.zero_mask, o, rr, c, gl);
}

template <int KP, int VPL>
__device__ __forceinline__ void ppr_slot(float *slots, uint32_t tile, const float *s, uint32_t gl)
{
    store_f32<VPL>(slots + (size_t)tile * KP + VPL * gl, s);
}

/* one group of KP/VPL lanes per tile, each lane VPL vectors with one
 * 16-byte access per edge; U edges' rows in flight per batch (one id per
 * lane); COHERENT: contributions read through L2 only (they are rewritten
 * inside the launch by the persistent kernel; the read-only path may keep
 * stale lines from an earlier iteration) */
template <int KP, int RS, class CT, int U, bool COHERENT>
__device__ __forceinline__ void ppr_gather_tiles(const PprArgs<CT> &a, const PprIter<CT> &it)
{
    typedef PprIO<CT, KP> IO;
    constexpr uint32_t VPL = IO::VPL;
    constexpr uint32_t LPE = KP / VPL;
    static_assert(U <= (int)LPE, "one id load per batch");
    static_assert(LPE >= 1 && LPE <= 32 && (32 % LPE) == 0, "lane groups tile the warp");
    const uint32_t lane = threadIdx.x & 31, gl = lane % LPE;
    const unsigned gmask = LPE == 32 ? 0xffffffffu : (((1u << LPE) - 1u) << (lane - gl));
    const uint32_t gid = (blockIdx.x * blockDim.x + threadIdx.x) / LPE;
    const uint32_t ngroups = (gridDim.x * blockDim.x) / LPE;
    for (uint32_t tile = gid; tile < a.ntiles; tile += ngroups)
    {
        const uint2 c0 = a.coord[tile], c1 = a.coord[tile + 1];
        const uint32_t i0 = c0.x, j0 = c0.y, i1 = c1.x, j1 = c1.y;
        /* rows rb .. rb+LPE-1, one per lane: end offset, seed index, 1 / out-degree */
        uint32_t rb = i0, w_end = 0, w_seed = NO_SEED;
        float w_inv = 0.0f;
        auto fetch = [&](uint32_t base) {
            rb = base;
            const uint32_t row = base + gl;
            w_end = a.E;
            w_seed = NO_SEED;
            w_inv = 0.0f;
            if (row < a.V)
            {
                w_end = a.off[row + 1];
                w_seed = a.seed_idx[row];
                w_inv = a.inv_deg[row];
            }
        };
        fetch(i0);
        /* row i0 began in an earlier tile when its first edge precedes j0 */
        const uint32_t start0 = i0 < a.V ? a.off[i0] : a.E;
        uint32_t r = i0;
        uint32_t re = __shfl_sync(gmask, w_end, 0, LPE);
        float acc[VPL];
#pragma unroll
        for (uint32_t k = 0; k < VPL; k++) acc[k] = 0.0f;
        /* finish row r (it ends in this tile) and move to r+1 */
        auto next_row = [&]() {
            const uint32_t k = r - rb;
            const uint32_t si = __shfl_sync(gmask, w_seed, k, LPE);
            const float inv = __shfl_sync(gmask, w_inv, k, LPE);
            if (r == i0 && start0 < j0)
                ppr_slot<KP, VPL>(a.head, tile, acc, gl);
            else
                ppr_finish<KP, RS, CT>(a, it, r, acc, si, inv, gl);
#pragma unroll
            for (uint32_t q = 0; q < VPL; q++) acc[q] = 0.0f;
            r++;
            if (r - rb >= LPE) fetch(r);
            re = __shfl_sync(gmask, w_end, r - rb, LPE);
        };
        /* the ids of a batch are loaded while the previous batch's rows are
         * in flight, so a batch waits for one memory latency, not two */
        uint32_t myid = 0;
        if (j0 < j1 && gl < min((uint32_t)U, j1 - j0)) myid = ldg_stream(a.adj + j0 + gl);
        for (uint32_t e = j0; e < j1; e += U)
        {
            const uint32_t nb = min((uint32_t)U, j1 - e);
            typename IO::Raw v[U];
#pragma unroll
            for (int i = 0; i < U; i++)
            {
                const uint32_t u = __shfl_sync(gmask, myid, i, LPE);
                if ((uint32_t)i < nb)
                    v[i] = COHERENT ? IO::load_cg(it.cin + (size_t)u * RS + VPL * gl)
                                    : IO::load(it.cin + (size_t)u * RS + VPL * gl);
            }
            const uint32_t en = e + U;
            myid = 0;
            if (en < j1 && gl < min((uint32_t)U, j1 - en)) myid = ldg_stream(a.adj + en + gl);
#pragma unroll
            for (int i = 0; i < U; i++)
            {
                if ((uint32_t)i < nb)
                {
                    /* rows ending before this edge, zero-degree rows included */
                    while (e + i >= re) next_row();
                    IO::add(acc, v[i]);
                }
            }
        }
        /* rows whose end items follow the tile's last edge */
        while (r < i1) next_row();
        /* row i1 continues in the next tile: leave what it gathered here */
        if (i1 < a.V && j1 > j0)
        {
            const uint32_t o = a.off[i1];
            if (o < j1) ppr_slot<KP, VPL>(a.tail, tile, acc, gl);
        }
    }
}

template <int KP, int RS, class CT, int U>
__global__ void __launch_bounds__(256) k_ppr_pull(PprArgs<CT> a)
{
    ppr_gather_tiles<KP, RS, CT, U, false>(a, PprIter<CT>{a.cin, a.cout, a.rank_mask});
}

/* finish the rows spanning tiles: the row that begins in tile t and is
 * still open at t's end (row coord[t+1].x) sums tail[t], the tails of the
 * tiles it crosses and the head of the tile where it ends, in tile order */
template <int KP, int RS, class CT>
__device__ __forceinline__ void ppr_fixup_tiles(const PprArgs<CT> &a, const PprIter<CT> &it)
{
    constexpr uint32_t VPL = PprIO<CT, KP>::VPL;
    constexpr uint32_t LPE = KP / VPL, B = 32 / VPL; /* tails in flight per lane: 32 floats */
    const uint32_t lane = threadIdx.x & 31, gl = lane % LPE;
    const uint32_t gid = (blockIdx.x * blockDim.x + threadIdx.x) / LPE;
    const uint32_t ngroups = (gridDim.x * blockDim.x) / LPE;
    for (uint32_t t = gid; t < a.ntiles; t += ngroups)
    {
        const uint32_t r = a.coord[t + 1].x;
        if (r >= a.V) continue;
        if ((((uint64_t)r + a.off[r]) >> a.tile_log2) != t) continue;
        /* the tile of the row's end item */
        const uint32_t t_last = (uint32_t)(((uint64_t)r + a.off[r + 1]) >> a.tile_log2);
        float tot[VPL];
        load_f32<VPL>(a.tail + (size_t)t * KP + VPL * gl, tot);
        for (uint32_t m = t + 1; m < t_last; m += B)
        {
            float v[B][VPL];
#pragma unroll
            for (uint32_t i = 0; i < B; i++)
                if (m + i < t_last) load_f32<VPL>(a.tail + (size_t)(m + i) * KP + VPL * gl, v[i]);
#pragma unroll
            for (uint32_t i = 0; i < B; i++)
                if (m + i < t_last)
#pragma unroll
                    for (uint32_t k = 0; k < VPL; k++) tot[k] += v[i][k];
        }
        float h[VPL];
        load_f32<VPL>(a.head + (size_t)t_last * KP + VPL * gl, h);
#pragma unroll
        for (uint32_t k = 0; k < VPL; k++) tot[k] += h[k];
        ppr_finish<KP, RS, CT>(a, it, r, tot, a.seed_idx[r], a.inv_deg[r], gl);
    }
}

template <int KP, int RS, class CT>
__global__ void __launch_bounds__(256) k_ppr_fixup(PprArgs<CT> a)
{
    ppr_fixup_tiles<KP, RS, CT>(a, PprIter<CT>{a.cin, a.cout, a.rank_mask});
}

/* every iteration in one cooperative launch: gather, grid barrier, fix-up
 * of the spanning rows, grid barrier.  The control block (GG_BAR_BYTES,
 * zeroed before the launch) holds the barrier; a barrier wait that runs out
 * sets *err and the launch ends (gg_set_barrier_limit_us). */
template <class CT>
struct PprLoop
{
    CT *cb0, *cb1;
    uint32_t iterations;
    char *ctl;
    unsigned int *err;
    unsigned long long limit_ns;
};

/* resident CTAs of the persistent kernel: its gather, fix-up and barrier
 * take ~120 registers per thread without spills, so 2 CTAs of 256 per SM
 * (3, with spills, measured the same) */
template <class CT> constexpr int ppr_persist_ctas() { return 2; }

template <int KP, class CT> constexpr int ppr_batch()
{
    constexpr int lpe = KP / ppr_vpl<CT, KP>();
    constexpr int umax = ppr_vpl<CT, KP>() == 2 ? 8 : (sizeof(CT) == 2 ? 6 : 4);
    return lpe < umax ? lpe : umax;
}

template <int KP, class CT, int U>
__global__ void __launch_bounds__(256, ppr_persist_ctas<CT>()) k_ppr_persist(const __grid_constant__ PprArgs<CT> a,
                                                                             const __grid_constant__ PprLoop<CT> L)
{
    unsigned int gen = 0;
    for (uint32_t i = 0; i < L.iterations; i++)
    {
        const PprIter<CT> it{(i & 1) ? L.cb1 : L.cb0, (i & 1) ? L.cb0 : L.cb1, i + 1 == L.iterations ? ~0ull : 0ull};
        ppr_gather_tiles<KP, KP, CT, U, true>(a, it);
        if (!grid_barrier(L.ctl, L.err, L.limit_ns, gen)) return;
        ppr_fixup_tiles<KP, KP, CT>(a, it);
        if (i + 1 < L.iterations && !grid_barrier(L.ctl, L.err, L.limit_ns, gen)) return;
    }
}

/* contributions of the seed vertices at iteration 0 (the rest is zero), and
 * their seed indices; rows of rs values, of which vectors in `fresh` are
 * written (all of them for gg_ppr; the newly admitted slots for the
 * server, whose other columns hold running vectors) */
template <class CT>
__global__ void k_ppr_seed_init(const uint32_t *__restrict__ seed_vertex, uint32_t nseeds,
                                const float *__restrict__ init, const uint32_t *__restrict__ outdeg, CT *cin,
                                uint32_t *seed_idx, uint32_t rs, unsigned long long fresh)
{
    const uint64_t n = (uint64_t)nseeds * (rs / 2);
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    {
        const uint32_t s = (uint32_t)(i / (rs / 2)), gl = (uint32_t)(i % (rs / 2));
        const uint32_t v = seed_vertex[s];
        if (gl == 0) seed_idx[v] = s;
        const uint32_t pair = (uint32_t)(fresh >> (2 * gl)) & 3u;
        if (!pair) continue;
        const uint32_t deg = outdeg[v];
        const float2 r = *reinterpret_cast<const float2 *>(init + (size_t)s * rs + 2 * gl);
        float c0 = 0.0f, c1 = 0.0f;
        if (deg)
        {
            const float fd = __uint2float_rn(deg);
            c0 = __fdiv_rn(r.x, fd);
            c1 = __fdiv_rn(r.y, fd);
        }
        CT *dst = cin + (size_t)v * rs + 2 * gl;
        /* only the fresh columns: the others belong to running vectors */
        if (pair & 1u) dst[0] = from_f32<CT>(c0);
        if (pair & 2u) dst[1] = from_f32<CT>(c1);
    }
}

/* inv[v] = 1 / out-degree (correctly rounded), 0 without out-edges */
__global__ void k_ppr_inv_deg(const uint32_t *__restrict__ outdeg, uint32_t V, float *inv)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
    {
        const uint32_t d = outdeg[v];
        inv[v] = d ? __frcp_rn(__uint2float_rn(d)) : 0.0f;
    }
}

gg_status ppr_inv_deg(gg_graph *g, cudaStream_t s, const float **out)
{
    void *inv;
    GG_CHECK(gg_work(g, 15, (size_t)g->V * 4 + 16, &inv));
    k_ppr_inv_deg<<<gg_sm_count() * 4, 256, 0, s>>>(g->out_deg, g->V, (float *)inv);
    GG_CUDA(cudaGetLastError());
    *out = (const float *)inv;
    return GG_OK;
}

template <class K>
int occupancy_grid(K kernel, int threads, size_t work_groups, int lanes_per_group)
{
    int bps = gg_occupancy((const void *)kernel, threads, 0);
    if (bps < 1) bps = 1;
    const size_t groups_per_block = (size_t)threads / lanes_per_group;
    const size_t need = (work_groups + groups_per_block - 1) / groups_per_block;
    const size_t cap = (size_t)gg_sm_count() * bps;
    const size_t g = need < cap ? need : cap;
    return (int)(g < 1 ? 1 : g);
}

template <int KP, class CT>
gg_status run_ppr(gg_graph *g, const gg_ppr_params *p, uint32_t nseedv, const uint32_t *d_seedv, const float *d_init,
                  const float *d_tele, uint32_t *d_seed_idx, float *d_rank, cudaStream_t s, gg_ppr_result &res,
                  std::vector<cudaEvent_t> &evs, void **ctl_out)
{
    constexpr int LPE = KP / PprIO<CT, KP>::VPL;
    constexpr int U = ppr_batch<KP, CT>();
    const uint32_t V = g->V;
    gg_tiles &t = g->ppr_tiles;
    const uint32_t tile = g->ppr_tile;
    if (t.coord && g->ppr_tiles_items != tile)
    {
        gg_dev_free(g, t.coord, ((size_t)t.ntiles + 1) * sizeof(uint2));
        t.coord = nullptr;
    }
    if (!t.coord)
    {
        const uint64_t nt = ((uint64_t)V + g->E + tile - 1) / tile;
        if (nt >= 0xffffffffull) return gg_fail(GG_ERR_INVALID, "graph too large for 32-bit tile ids");
        t.ntiles = (uint32_t)(nt ? nt : 1);
        GG_CHECK(gg_dev_alloc(g, (void **)&t.coord, ((size_t)t.ntiles + 1) * sizeof(uint2)));
        GG_CHECK(gg_launch_tile_coords(g->in_off, V, g->E, t.ntiles, t.coord, s, tile));
        g->ppr_tiles_items = tile;
        res.launches++;
    }
    void *c0, *c1, *slots;
    GG_CHECK(gg_work(g, 16, (size_t)V * KP * sizeof(CT), &c0));
    GG_CHECK(gg_work(g, 17, (size_t)V * KP * sizeof(CT), &c1));
    GG_CHECK(gg_work(g, 18, (size_t)t.ntiles * KP * sizeof(float) * 2, &slots));
    GG_CUDA(cudaMemsetAsync(c0, 0, (size_t)V * KP * sizeof(CT), s));
    GG_CUDA(cudaMemsetAsync(d_seed_idx, 0xff, (size_t)V * sizeof(uint32_t), s));
    k_ppr_seed_init<CT><<<gg_sm_count() * 2, 256, 0, s>>>(d_seedv, nseedv, d_init, g->out_deg, (CT *)c0, d_seed_idx,
                                                          KP, ~0ull);
    res.launches++;

    PprArgs<CT> a;
    a.off = g->in_off; a.adj = g->in_adj; a.seed_idx = d_seed_idx;
    GG_CHECK(ppr_inv_deg(g, s, &a.inv_deg));
    res.launches++;
    a.coord = t.coord; a.ntiles = t.ntiles; a.V = V; a.E = g->E; a.tile_log2 = (uint32_t)__builtin_ctz(tile);
    a.rank = d_rank; a.rank_mask = 0; a.zero_mask = 0;
    a.tele = d_tele; a.damp = p->damp;
    a.head = (float *)slots;
    a.tail = (float *)slots + (size_t)t.ntiles * KP;
    CT *cb[2] = {(CT *)c0, (CT *)c1};
    if (!p->profile)
    {
        /* all iterations in one cooperative launch: every block resident */
        const int per_sm = gg_occupancy((const void *)k_ppr_persist<KP, CT, U>, 256, 0);
        if (per_sm < 1) return gg_fail(GG_ERR_CUDA, "k_ppr_persist cannot be resident");
        const size_t groups_per_block = 256 / LPE;
        const size_t need = ((size_t)t.ntiles + groups_per_block - 1) / groups_per_block;
        const size_t cap = (size_t)gg_sm_count() * (size_t)per_sm;
        const int grid = (int)(need < cap ? (need ? need : 1) : cap);
        void *ctl;
        GG_CHECK(gg_work(g, 30, GG_BAR_BYTES, &ctl));
        GG_CUDA(cudaMemsetAsync(ctl, 0, GG_BAR_BYTES, s));
        PprLoop<CT> L;
        L.cb0 = cb[0]; L.cb1 = cb[1]; L.iterations = p->iterations;
        L.ctl = (char *)ctl; L.err = (unsigned int *)ctl; L.limit_ns = gg_barrier_limit_ns();
        void *args[] = {&a, &L};
        GG_CUDA(cudaLaunchCooperativeKernel((const void *)k_ppr_persist<KP, CT, U>, dim3(grid), dim3(256), args, 0, s));
        res.launches++;
        res.gather_launches = p->iterations;
        res.persistent = 1;
        *ctl_out = ctl;
        GG_CUDA(cudaGetLastError());
        return GG_OK;
    }
    const int grid = occupancy_grid(k_ppr_pull<KP, KP, CT, U>, 256, t.ntiles, LPE);
    const int fgrid = occupancy_grid(k_ppr_fixup<KP, KP, CT>, 256, t.ntiles, LPE);
    for (uint32_t it = 0; it < p->iterations; it++)
    {
        a.cin = cb[it & 1];
        a.cout = cb[(it + 1) & 1];
        a.rank_mask = it + 1 == p->iterations ? ~0ull : 0ull;
        if (p->profile)
        {
            cudaEvent_t e;
            GG_CHECK(gg_event_at(g, (uint32_t)evs.size(), &e));
            GG_CUDA(cudaEventRecord(e, s));
            evs.push_back(e);
        }
        k_ppr_pull<KP, KP, CT, U><<<grid, 256, 0, s>>>(a);
        if (p->profile)
        {
            cudaEvent_t e;
            GG_CHECK(gg_event_at(g, (uint32_t)evs.size(), &e));
            GG_CUDA(cudaEventRecord(e, s));
            evs.push_back(e);
        }
        k_ppr_fixup<KP, KP, CT><<<fgrid, 256, 0, s>>>(a);
        res.launches += 2;
        res.gather_launches++;
    }
    GG_CUDA(cudaGetLastError());
    return GG_OK;
}

} // namespace

/* ---- one iteration on caller-held state (the server's continuous batch) ----- */

namespace {

template <int KP, class CT>
gg_status round_run(gg_graph *g, const gg_ppr_round_args &r, cudaStream_t s)
{
    constexpr int LPE = KP / PprIO<CT, KP>::VPL;
    constexpr int U = ppr_batch<KP, CT>();
    gg_tiles &t = g->ppr_tiles;
    PprArgs<CT> a;
    a.off = g->in_off; a.adj = g->in_adj; a.seed_idx = r.seed_idx;
    void *inv;
    GG_CHECK(gg_work(g, 15, (size_t)g->V * 4 + 16, &inv)); /* filled by gg_ppr_round_prepare */
    a.inv_deg = (const float *)inv;
    a.coord = t.coord; a.ntiles = t.ntiles; a.V = g->V; a.E = g->E;
    a.tile_log2 = (uint32_t)__builtin_ctz(g->ppr_tiles_items);
    a.cin = (const CT *)r.cin; a.cout = (CT *)r.cout; a.rank = r.rank;
    a.rank_mask = r.rank_mask; a.zero_mask = r.zero_mask;
    a.tele = r.tele; a.damp = r.damp;
    a.head = r.slots;
    a.tail = r.slots + (size_t)t.ntiles * KP;
    const int grid = occupancy_grid(k_ppr_pull<KP, 64, CT, U>, 256, t.ntiles, LPE);
    const int fgrid = occupancy_grid(k_ppr_fixup<KP, 64, CT>, 256, t.ntiles, LPE);
    k_ppr_pull<KP, 64, CT, U><<<grid, 256, 0, s>>>(a);
    k_ppr_fixup<KP, 64, CT><<<fgrid, 256, 0, s>>>(a);
    GG_CUDA(cudaGetLastError());
    return GG_OK;
}

} // namespace

gg_status gg_ppr_round_prepare(gg_graph *g, uint32_t rs, int bf16, void **cb0, void **cb1, float **slots,
                               cudaStream_t s)
{
    gg_tiles &t = g->ppr_tiles;
    const uint32_t tile = g->ppr_tile;
    const uint32_t V = g->V;
    if (t.coord && g->ppr_tiles_items != tile)
    {
        gg_dev_free(g, t.coord, ((size_t)t.ntiles + 1) * sizeof(uint2));
        t.coord = nullptr;
    }
    if (!t.coord)
    {
        const uint64_t nt = ((uint64_t)V + g->E + tile - 1) / tile;
        if (nt >= 0xffffffffull) return gg_fail(GG_ERR_INVALID, "graph too large for 32-bit tile ids");
        t.ntiles = (uint32_t)(nt ? nt : 1);
        GG_CHECK(gg_dev_alloc(g, (void **)&t.coord, ((size_t)t.ntiles + 1) * sizeof(uint2)));
        GG_CHECK(gg_launch_tile_coords(g->in_off, V, g->E, t.ntiles, t.coord, s, tile));
        g->ppr_tiles_items = tile;
    }
    const size_t cb = (size_t)V * rs * (bf16 ? 2 : 4);
    GG_CHECK(gg_work(g, 16, cb, cb0));
    GG_CHECK(gg_work(g, 17, cb, cb1));
    GG_CHECK(gg_work(g, 18, (size_t)t.ntiles * rs * sizeof(float) * 2, (void **)slots));
    GG_CUDA(cudaMemsetAsync(*cb0, 0, cb, s));
    GG_CUDA(cudaMemsetAsync(*cb1, 0, cb, s));
    const float *inv;
    GG_CHECK(ppr_inv_deg(g, s, &inv));
    return GG_OK;
}

gg_status gg_ppr_round_seed(gg_graph *g, uint32_t rs, int bf16, void *cin, const uint32_t *d_seedv, uint32_t nseedv,
                            const float *d_init, uint32_t *d_seed_idx, unsigned long long fresh, cudaStream_t s)
{
    if (!nseedv) return GG_OK;
    if (bf16)
        k_ppr_seed_init<__nv_bfloat16><<<gg_sm_count() * 2, 256, 0, s>>>(d_seedv, nseedv, d_init, g->out_deg,
                                                                         (__nv_bfloat16 *)cin, d_seed_idx, rs, fresh);
    else
        k_ppr_seed_init<float><<<gg_sm_count() * 2, 256, 0, s>>>(d_seedv, nseedv, d_init, g->out_deg, (float *)cin,
                                                                 d_seed_idx, rs, fresh);
    GG_CUDA(cudaGetLastError());
    return GG_OK;
}

gg_status gg_ppr_round(gg_graph *g, const gg_ppr_round_args &r, cudaStream_t s)
{
    if (r.bf16)
        return r.kp == 16 ? round_run<16, __nv_bfloat16>(g, r, s)
               : r.kp == 32 ? round_run<32, __nv_bfloat16>(g, r, s) : round_run<64, __nv_bfloat16>(g, r, s);
    return r.kp == 16 ? round_run<16, float>(g, r, s) : r.kp == 32 ? round_run<32, float>(g, r, s)
                                                                : round_run<64, float>(g, r, s);
}

extern "C" gg_status gg_ppr(gg_graph *g, const gg_ppr_params *p, const uint32_t *seed_off, const uint32_t *seeds,
                            float *ranks, gg_ppr_result *r, void *stream)
{
    GgRange range("gg_ppr");
    if (!g || !p || !seed_off) return gg_fail(GG_ERR_INVALID, "NULL argument");
    const uint32_t K = p->num_vectors;
    if (K < 1 || K > 64) return gg_fail(GG_ERR_INVALID, "num_vectors must be 1..64");
    if (p->iterations < 1) return gg_fail(GG_ERR_INVALID, "iterations must be at least 1");
    if (p->storage != GG_STORE_F32 && p->storage != GG_STORE_BF16)
        return gg_fail(GG_ERR_INVALID, "batched PageRank stores FP32 or BF16 contributions");
    if (!g->in_off || !g->out_deg) return gg_fail(GG_ERR_INVALID, "batched PageRank needs GG_MAP_IN");
    if (seed_off[0] != 0) return gg_fail(GG_ERR_INVALID, "seed_off[0] must be 0");
    for (uint32_t k = 0; k < K; k++)
        if (seed_off[k + 1] < seed_off[k]) return gg_fail(GG_ERR_INVALID, "seed_off must be non-decreasing");
    const uint32_t nseeds = seed_off[K];
    if (nseeds && !seeds) return gg_fail(GG_ERR_INVALID, "NULL seeds");
    const uint32_t V = g->V;
    for (uint32_t i = 0; i < nseeds; i++)
        if (seeds[i] >= V) return gg_fail(GG_ERR_INVALID, "seed vertex out of range");
    const uint32_t KP = K <= 16 ? 16 : (K <= 32 ? 32 : 64);
    cudaStream_t s = gg_stream(g, stream);
    gg_tune_lookup(g, s);
    gg_ppr_result res;
    memset(&res, 0, sizeof(res));
    res.padded_vectors = KP;

    /* seed vertices, each with its initial-rank and teleport rows */
    std::vector<uint32_t> verts;
    std::unordered_map<uint32_t, uint32_t> index;
    for (uint32_t i = 0; i < nseeds; i++)
        if (index.emplace(seeds[i], (uint32_t)verts.size()).second) verts.push_back(seeds[i]);
    const uint32_t nv = (uint32_t)verts.size();
    std::vector<double> share((size_t)nv * KP, 0.0);
    for (uint32_t k = 0; k < K; k++)
    {
        const uint32_t n = seed_off[k + 1] - seed_off[k];
        for (uint32_t i = seed_off[k]; i < seed_off[k + 1]; i++)
            share[(size_t)index[seeds[i]] * KP + k] += 1.0 / (double)n;
    }
    std::vector<float> tables((size_t)nv * KP * 2);
    for (size_t i = 0; i < share.size(); i++)
    {
        tables[i] = (float)share[i];
        tables[share.size() + i] = (float)((1.0 - (double)p->damp) * share[i]);
    }
    void *d_seedv = nullptr, *d_tab = nullptr, *d_idx, *d_rank;
    if (V > 0)
    {
        GG_CHECK(gg_work(g, 19, ((size_t)nv + 1) * 4, &d_seedv));
        GG_CHECK(gg_work(g, 20, (tables.size() + 4) * sizeof(float), &d_tab));
        GG_CHECK(gg_work(g, 21, (size_t)V * 4, &d_idx));
        GG_CHECK(gg_work(g, 22, (size_t)V * KP * sizeof(float), &d_rank));
        if (nv)
        {
            GG_CUDA(cudaMemcpyAsync(d_seedv, verts.data(), (size_t)nv * 4, cudaMemcpyHostToDevice, s));
            GG_CUDA(cudaMemcpyAsync(d_tab, tables.data(), tables.size() * sizeof(float), cudaMemcpyHostToDevice, s));
        }
        std::vector<cudaEvent_t> evs;
        void *ctl = nullptr;
        const float *d_init = (const float *)d_tab, *d_tele = (const float *)d_tab + (size_t)nv * KP;
        gg_status st;
#define GG_PPR_RUN(KPV, CTV)                                                                                          \
    run_ppr<KPV, CTV>(g, p, nv, (const uint32_t *)d_seedv, d_init, d_tele, (uint32_t *)d_idx, (float *)d_rank, s,     \
                      res, evs, &ctl)
        if (p->storage == GG_STORE_BF16)
            st = KP == 16 ? GG_PPR_RUN(16, __nv_bfloat16) : KP == 32 ? GG_PPR_RUN(32, __nv_bfloat16) : GG_PPR_RUN(64, __nv_bfloat16);
        else
            st = KP == 16 ? GG_PPR_RUN(16, float) : KP == 32 ? GG_PPR_RUN(32, float) : GG_PPR_RUN(64, float);
#undef GG_PPR_RUN
        if (st != GG_OK) return st;
        GG_CHECK(gg_wait(s)); /* bounded, before a copy to pageable memory */
        if (ranks)
            GG_CUDA(cudaMemcpy2DAsync(ranks, (size_t)K * sizeof(float), d_rank, (size_t)KP * sizeof(float),
                                      (size_t)K * sizeof(float), V, cudaMemcpyDeviceToHost, s));
        uint32_t *h_err = nullptr;
        if (ctl)
        {
            GG_CHECK(gg_pinned(g, 64, (void **)&h_err));
            GG_CUDA(cudaMemcpyAsync(h_err, ctl, 4, cudaMemcpyDeviceToHost, s));
        }
        GG_CHECK(gg_wait(s));
        if (h_err && *h_err) return gg_fail(GG_ERR_KERNEL, "batched PageRank grid barrier timed out");
        for (size_t i = 0; i + 1 < evs.size(); i += 2) res.gather_ms += gg_event_ms(evs[i], evs[i + 1]);
        g->ppr_ranks = (const float *)d_rank;
        g->ppr_stride = KP;
    }
    if (r) *r = res;
    return GG_OK;
}

extern "C" const float *gg_ppr_device_ranks(const gg_graph *g, uint32_t *stride)
{
    if (!g) return nullptr;
    if (stride) *stride = g->ppr_stride;
    return g->ppr_ranks;
}
