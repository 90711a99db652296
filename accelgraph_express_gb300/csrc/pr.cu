/*
 * PageRank on CSR, all fourteen variants of the reference's dispatcher
 * (02_capi_graph/src/algorithms/capi/pageRank.c:874-939), on one GPU.
 *
 * Topology-driven pull (modes 0, 2, 4, 9-13): one launch per iteration of
 * the merge-path tile gather over the CSC, fused with the reference's update
 * pass (pageRank.c:1055-1069) and with the next iteration's contribution
 * pass (pageRank.c:1026-1033):
 *     sum      = sum over in-edges (u,v) of contrib[u]      (FP32 or u64)
 *     rank'    = 0.15 + 0.85*sum
 *     error   += |rank' - rank| / V   (FP64),  active += (|.| >= epsilon)
 *     contrib' = rank' / outdeg(v)    (0 when outdeg is 0)
 * Contributions are double-buffered; the FP64 residual and active count go
 * to a per-iteration record, and every launch of iteration k returns at once
 * when iteration k-1 left no active vertex, so all iterations are queued
 * without a host round trip and the host reads the records once.
 *
 * Push (modes 1, 3, 5): the same tiles over the out-CSR scatter with
 * atomics into next[], then a vertex pass does the update.
 * Data-driven (modes 6, 7, 8): worklist variants (pageRank.c:2810-3300).
 *
 * Storage: contributions in FP32, BF16 or FP16 (FP32 accumulation), or in
 * the fixed-point / quantised integer formats summed exactly in 64 bits.
 */
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "gg_device.cuh"

namespace {

using namespace gg;

/* per-iteration record written by the kernels */
struct IterRec
{
    double err;
    uint32_t active;
    uint32_t maxbits;  /* max contribution (float bits) for the quantised modes */
};

/* ---- contribution formats --------------------------------------------------- */

enum Kind { K_F32, K_BF16, K_F16, K_FX64, K_FX32, K_FX16, K_FX8, K_Q32, K_Q16, K_Q8, K_Q8Z };

template <int K> struct Fmt;
template <> struct Fmt<K_F32> { typedef float CT; typedef float Acc; static constexpr bool quant = false; };
template <> struct Fmt<K_BF16> { typedef __nv_bfloat16 CT; typedef float Acc; static constexpr bool quant = false; };
template <> struct Fmt<K_F16> { typedef __half CT; typedef float Acc; static constexpr bool quant = false; };
template <> struct Fmt<K_FX64> { typedef unsigned long long CT; typedef unsigned long long Acc; static constexpr bool quant = false; };
template <> struct Fmt<K_FX32> { typedef uint32_t CT; typedef unsigned long long Acc; static constexpr bool quant = false; };
template <> struct Fmt<K_FX16> { typedef uint16_t CT; typedef unsigned long long Acc; static constexpr bool quant = false; };
template <> struct Fmt<K_FX8> { typedef uint8_t CT; typedef unsigned long long Acc; static constexpr bool quant = false; };
template <> struct Fmt<K_Q32> { typedef uint32_t CT; typedef unsigned long long Acc; static constexpr bool quant = true; static constexpr int bits = 32; };
template <> struct Fmt<K_Q16> { typedef uint16_t CT; typedef unsigned long long Acc; static constexpr bool quant = true; static constexpr int bits = 16; };
template <> struct Fmt<K_Q8> { typedef uint8_t CT; typedef unsigned long long Acc; static constexpr bool quant = true; static constexpr int bits = 8; };
/* push variant of the quantised mode: 8 bits with a zero point, FP32 scatter */
template <> struct Fmt<K_Q8Z> { typedef uint8_t CT; typedef float Acc; static constexpr bool quant = true; static constexpr int bits = 8; };

/* stored contribution of a vertex from its new rank (pageRank.c:1028-1031
 * and the fixed-point forms at :1373, :1553, :1730, :1911) */
template <int K>
__device__ __forceinline__ typename Fmt<K>::CT encode(float c, uint32_t deg)
{
    if constexpr (K == K_F32 || K == K_BF16 || K == K_F16)
        return from_f32<typename Fmt<K>::CT>(c);
    else if constexpr (K == K_FX64)
        return deg ? fx64_from_double((double)c) : 0ull;
    else if constexpr (K == K_FX32)
        return deg ? fx_from_float(c, 65536.0, 0xffffffffu) : 0u;
    else if constexpr (K == K_FX16)
        return (uint16_t)(deg ? fx_from_float(c, 4096.0, 0xffffu) : 0u);
    else if constexpr (K == K_FX8)
        return (uint8_t)(deg ? fx_from_float(c, 64.0, 0xffu) : 0u);
    else
        return 0; /* quantised formats are written by k_quantize */
}

template <int K>
__device__ __forceinline__ typename Fmt<K>::Acc decode(typename Fmt<K>::CT x)
{
    if constexpr (K == K_F32 || K == K_BF16 || K == K_F16)
        return to_f32(x);
    else
        return (unsigned long long)x;
}

/* rank' from the gathered sum (pageRank.c:1057, :1400, :1581, :1758, :1939, :2252) */
template <int K>
__device__ __forceinline__ float next_rank(float base, float damp, typename Fmt<K>::Acc sum, float qscale)
{
    if constexpr (K == K_F32 || K == K_BF16 || K == K_F16)
        return __fadd_rn(base, __fmul_rn(damp, sum));
    else if constexpr (K == K_FX64)
        return __double2float_rn(__dadd_rn((double)base, __dmul_rn((double)damp, fx64_to_double(sum))));
    else if constexpr (K == K_FX32)
        return __fadd_rn(base, __fmul_rn(damp, fx_to_float(sum, 1.0 / 65536.0)));
    else if constexpr (K == K_FX16)
        return __fadd_rn(base, __fmul_rn(damp, fx_to_float(sum, 1.0 / 4096.0)));
    else if constexpr (K == K_FX8)
        return __fadd_rn(base, __fmul_rn(damp, fx_to_float(sum, 1.0 / 64.0)));
    else
        return __fadd_rn(base, __fmul_rn(damp, __fmul_rn(qscale, __ull2float_rn(sum))));
}

__device__ __forceinline__ float contrib_of(float rank, uint32_t deg)
{
    return deg ? __fdiv_rn(rank, __uint2float_rn(deg)) : 0.0f;
}

/* quantisation, same arithmetic as the oracle's orc_quant_* */
__device__ __forceinline__ float quant_scale(uint32_t maxbits, int bits)
{
    float mx = __uint_as_float(maxbits);
    if (!(mx > 0.0f)) return 0.0f;
    double levels = (double)((1ull << bits) - 1);
    return __double2float_rn(__ddiv_rn((double)mx, levels));
}
__device__ __forceinline__ uint32_t quantize(float x, float scale, uint32_t zero, int bits)
{
    double maxq = (double)((1ull << bits) - 1);
    if (scale == 0.0f) return zero;
    double t = floor(__dadd_rn(__ddiv_rn((double)x, (double)scale), 0.5)) + (double)zero;
    if (t < 0.0) return 0u;
    if (t > maxq) return (uint32_t)maxq;
    return (uint32_t)t;
}
__device__ __forceinline__ uint32_t quant_zero(uint32_t maxbits, float scale, int bits)
{
    double maxq = (double)((1ull << bits) - 1);
    if (scale == 0.0f) return 0u;
    double t = floor(__dsub_rn(maxq, __ddiv_rn((double)__uint_as_float(maxbits), (double)scale)) + 0.5);
    if (t < 0.0) return 0u;
    if (t > maxq) return (uint32_t)maxq;
    return (uint32_t)t;
}

/* block max of non-negative floats as their bit patterns, then one atomic */
template <int NT>
__device__ __forceinline__ void block_max_bits(uint32_t v, uint32_t *dst)
{
    __shared__ uint32_t sm[NT / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_down_sync(0xffffffffu, v, o));
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sm[w] = v;
    __syncthreads();
    if (w == 0)
    {
        v = l < NT / 32 ? sm[l] : 0u;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_down_sync(0xffffffffu, v, o));
        if (l == 0 && v) atomicMax(dst, v);
    }
    __syncthreads();
}

struct PrCommon
{
    float *rank;
    const uint32_t *outdeg;
    uint32_t V;
    float base, damp;
    float eps_f;       /* smallest float e with (double)e >= epsilon */
    float eps_fl;      /* largest float e with (double)e <= epsilon */
    IterRec *rec;      /* records of this run */
    uint32_t it;       /* iteration index of this launch */
    __device__ __forceinline__ bool skip() const { return it > 0 && rec[it - 1].active == 0u; }
    /* pageRank.c:1057-1067: |rank' - rank| is a float difference, exact in
     * FP64; the FP64 sum of the differences is divided by V once on the host
     * (the reference divides each term), and `error >= epsilon` is the same
     * test as e >= eps_f in FP32, so no FP64 division or compare runs per
     * vertex (FP64 is 1/64 of the FP32 rate here) */
    __device__ __forceinline__ void update(uint32_t r, float nr, double &err, uint32_t &act) const
    {
        float pr = rank[r];
        rank[r] = nr;
        float e = fabsf(__fsub_rn(nr, pr));
        err += (double)e;
        if (e >= eps_f) act++;
    }
    __device__ __forceinline__ void update_pre(uint32_t r, float nr, float pr, double &err, uint32_t &act) const
    {
        rank[r] = nr;
        float e = fabsf(__fsub_rn(nr, pr));
        err += (double)e;
        if (e >= eps_f) act++;
    }
    __device__ __forceinline__ void reduce(double err, uint32_t act) const
    {
        if (err != 0.0) atomicAdd(&rec[it].err, err);
        if (act) atomicAdd(&rec[it].active, act);
    }
    __device__ __forceinline__ void warp_reduce(double err, uint32_t act) const
    {
        warp_reduce_to(err, act, &rec[it].err, &rec[it].active);
    }
};

/* ---- pull: gather + fused update ------------------------------------------------ */

template <int K>
struct PullOp : PrCommon
{
    typedef typename Fmt<K>::Acc Acc;
    typedef typename Fmt<K>::CT CT;
    const CT *cin;
    CT *cout;
    float *cf;         /* float contributions (quantised modes) */
    uint32_t tmax = 0; /* this thread's largest new contribution (quantised modes) */

    struct RowPre { float rank; uint32_t deg; };
    static constexpr uint32_t PRE_WORDS = 2;
    __device__ __forceinline__ Acc load1(uint32_t, uint32_t u) const { return decode<K>(cin[u]); }
    __device__ __forceinline__ RowPre prefetch(uint32_t r) const { return RowPre{rank[r], outdeg[r]}; }
    __device__ __forceinline__ void stage(uint32_t i0, uint32_t n, uint32_t lane, uint32_t *s, uint32_t stride) const
    {
        stage_words(s, reinterpret_cast<const uint32_t *>(rank), i0, n, lane);
        stage_words(s + stride, outdeg, i0, n, lane);
    }
    __device__ __forceinline__ RowPre unstage(uint32_t, const uint32_t *s, uint32_t j, uint32_t stride) const
    {
        return RowPre{__uint_as_float(s[j]), s[stride + j]};
    }
    __device__ __forceinline__ void finish(uint32_t r, Acc sum, const RowPre &pre, double &err, uint32_t &act)
    {
        float qscale = 0.0f;
        if constexpr (Fmt<K>::quant) qscale = quant_scale(rec[it].maxbits, Fmt<K>::bits);
        float nr = next_rank<K>(base, damp, sum, qscale);
        update_pre(r, nr, pre.rank, err, act);
        const uint32_t d = pre.deg;
        float c = contrib_of(nr, d);
        if constexpr (Fmt<K>::quant)
        {
            cf[r] = c;
            tmax = max(tmax, __float_as_uint(c));
        }
        else
            cout[r] = encode<K>(c, d);
    }
    __device__ __forceinline__ void warp_end(double err, uint32_t act)
    {
        warp_reduce(err, act);
        if constexpr (Fmt<K>::quant) warp_max_to(tmax, &rec[it + 1].maxbits);
    }
};

template <int K>
__global__ void __launch_bounds__(GG_TILE_NT) k_pr_pull(const uint32_t *__restrict__ off,
                                                        const uint32_t *__restrict__ adj, const uint2 *__restrict__ coord,
                                                        uint32_t ntiles, typename Fmt<K>::Acc *g_acc, PullOp<K> op)
{
    if (op.skip()) return;
    warp_pull<GG_TILE_IPT, GG_TILE_WARPS>(off, adj, op.V, coord, ntiles, g_acc, op);
}

template <int K>
__global__ void __launch_bounds__(256) k_pr_pull_fixup(const uint32_t *__restrict__ off, const uint2 *__restrict__ coord,
                                                       uint32_t ntiles, typename Fmt<K>::Acc *g_acc, PullOp<K> op)
{
    if (op.skip()) return;
    warp_pull_fixup(off, op.V, coord, ntiles, GG_TILE_ITEMS, g_acc, op);
}

/* ---- init, quantise, finalise --------------------------------------------------- */

template <int K>
__global__ void k_pr_init(float *__restrict__ rank, const uint32_t *__restrict__ outdeg, uint32_t V, float init,
                          typename Fmt<K>::CT *cout, float *cf, IterRec *rec)
{
    uint32_t tmax = 0;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
    {
        rank[v] = init;
        uint32_t d = outdeg[v];
        float c = contrib_of(init, d);
        if constexpr (Fmt<K>::quant)
        {
            cf[v] = c;
            tmax = max(tmax, __float_as_uint(c));
        }
        else if (cout)
            cout[v] = encode<K>(c, d);
    }
    if constexpr (Fmt<K>::quant) block_max_bits<256>(tmax, &rec[0].maxbits);
}

/* q[v] = quantize(contrib[v]) with the scale of iteration `it`
 * (pageRank.c:2212-2226); bits = 8 with a zero point is the push variant
 * (pageRank.c:2727-2737) */
template <class QT>
__global__ void k_quantize(const float *__restrict__ cf, QT *__restrict__ q, uint32_t V, int bits, int with_zero,
                           IterRec *rec, uint32_t it, uint32_t *zero_out)
{
    if (it > 0 && rec[it - 1].active == 0u) return;
    const uint32_t mb = rec[it].maxbits;
    const float scale = quant_scale(mb, bits);
    const uint32_t zero = with_zero ? quant_zero(mb, scale, bits) : 0u;
    if (zero_out && blockIdx.x == 0 && threadIdx.x == 0) zero_out[it] = zero;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
        q[v] = (QT)quantize(cf[v], scale, zero, bits);
}

/* final normalisation and sum (pageRank.c:1080-1085) */
__global__ void k_pr_finalize(float *__restrict__ rank, uint32_t V, int divide, double *sum)
{
    double s = 0.0;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
    {
        float r = rank[v];
        if (divide)
        {
            r = __fdiv_rn(r, __uint2float_rn(V));
            rank[v] = r;
        }
        s += (double)r;
    }
    uint32_t dummy = 0;
    block_sum2<256>(s, dummy);
    if (threadIdx.x == 0 && s != 0.0) atomicAdd(sum, s);
}

/* ---- push: scatter + vertex update ---------------------------------------------- */

template <int K>
__global__ void __launch_bounds__(GG_TILE_NT) k_pr_push_f(const uint32_t *__restrict__ off, const uint32_t *__restrict__ adj,
                                                          const uint2 *__restrict__ coord, uint32_t ntiles, uint32_t V,
                                                          const typename Fmt<K>::CT *cin, float *next,
                                                          IterRec *rec, uint32_t it)
{
    if (it > 0 && rec[it - 1].active == 0u) return;
    struct Op
    {
        typedef float RowVal;
        const typename Fmt<K>::CT *cin;
        float *next;
        __device__ __forceinline__ float row_value(uint32_t r) const { return to_f32(cin[r]); }
        __device__ __forceinline__ void scatter(float rv, uint32_t, uint32_t dst) const { atomicAdd(&next[dst], rv); }
    } op{cin, next};
    warp_push<GG_TILE_IPT, GG_TILE_WARPS>(off, adj, V, coord, ntiles, op);
}

__global__ void __launch_bounds__(GG_TILE_NT) k_pr_push_fx64(const uint32_t *__restrict__ off, const uint32_t *__restrict__ adj,
                                                             const uint2 *__restrict__ coord, uint32_t ntiles, uint32_t V,
                                                             const unsigned long long *cin, unsigned long long *next,
                                                             IterRec *rec, uint32_t it)
{
    if (it > 0 && rec[it - 1].active == 0u) return;
    struct Op
    {
        typedef unsigned long long RowVal;
        const unsigned long long *cin;
        unsigned long long *next;
        __device__ __forceinline__ unsigned long long row_value(uint32_t r) const { return cin[r]; }
        __device__ __forceinline__ void scatter(unsigned long long rv, uint32_t, uint32_t dst) const
        {
            atomicAdd(&next[dst], rv);
        }
    } op{cin, next};
    warp_push<GG_TILE_IPT, GG_TILE_WARPS>(off, adj, V, coord, ntiles, op);
}

__global__ void __launch_bounds__(GG_TILE_NT) k_pr_push_q(const uint32_t *__restrict__ off, const uint32_t *__restrict__ adj,
                                                          const uint2 *__restrict__ coord, uint32_t ntiles, uint32_t V,
                                                          const uint8_t *q, const uint32_t *zeros, float *next,
                                                          IterRec *rec, uint32_t it)
{
    if (it > 0 && rec[it - 1].active == 0u) return;
    struct Op
    {
        typedef float RowVal;
        const uint8_t *q;
        float scale;
        uint32_t zero;
        float *next;
        /* pageRank.c:2753: scale * (q - zero) */
        __device__ __forceinline__ float row_value(uint32_t r) const
        {
            return __fmul_rn(scale, (float)((long long)q[r] - (long long)zero));
        }
        __device__ __forceinline__ void scatter(float rv, uint32_t, uint32_t dst) const { atomicAdd(&next[dst], rv); }
    } op{q, quant_scale(rec[it].maxbits, 8), zeros[it], next};
    warp_push<GG_TILE_IPT, GG_TILE_WARPS>(off, adj, V, coord, ntiles, op);
}

/* vertex update after a push (pageRank.c:2067-2081) */
template <int K>
__global__ void k_pr_push_update(PrCommon c, typename Fmt<K>::Acc *next, typename Fmt<K>::CT *cout, float *cf)
{
    if (c.skip()) return;
    double err = 0.0;
    uint32_t act = 0, tmax = 0;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < c.V; v += gridDim.x * blockDim.x)
    {
        typename Fmt<K>::Acc s = next[v];
        next[v] = 0;
        float nr;
        if constexpr (K == K_FX64)
            nr = next_rank<K_FX64>(c.base, c.damp, s, 0.0f);
        else
            nr = __fadd_rn(c.base, __fmul_rn(c.damp, (float)s));
        c.update(v, nr, err, act);
        uint32_t d = c.outdeg[v];
        float ctb = contrib_of(nr, d);
        if constexpr (K == K_Q8Z)
        {
            cf[v] = ctb;
            tmax = max(tmax, __float_as_uint(ctb));
        }
        else
            cout[v] = encode<K>(ctb, d);
    }
    if constexpr (K == K_Q8Z) block_max_bits<256>(tmax, &c.rec[c.it + 1].maxbits);
    block_sum2<256>(err, act);
    if (threadIdx.x == 0) c.reduce(err, act);
}

/* ---- data-driven variants (pageRank.c:2810-3300) -------------------------------- */

__global__ void k_dd_contrib(const float *__restrict__ rank, const uint32_t *__restrict__ outdeg, float *cf, uint32_t V,
                             IterRec *rec, uint32_t it)
{
    if (it > 0 && rec[it - 1].active == 0u) return;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
        cf[v] = contrib_of(rank[v], outdeg[v]);
}

/* data-driven pull: only worklist vertices update; a vertex that moved by at
 * least epsilon keeps its new rank and activates its out-neighbours */
struct DdPullOp : PrCommon
{
    typedef float Acc;
    const float *cf;
    const uint8_t *wl_curr;
    uint8_t *wl_next;
    const uint32_t *out_off, *out_adj;
    struct RowPre { float rank; uint32_t on; };
    static constexpr uint32_t PRE_WORDS = 2;
    __device__ __forceinline__ float load1(uint32_t, uint32_t u) const { return cf[u]; }
    __device__ __forceinline__ RowPre prefetch(uint32_t r) const { return RowPre{rank[r], wl_curr[r]}; }
    /* the flag bytes travel as the aligned 4-byte words holding them: word
     * c of the second plane holds rows (i0 & ~3) + 4c .. +3 (the worklists
     * are allocated with 16 bytes of slack past V) */
    __device__ __forceinline__ void stage(uint32_t i0, uint32_t n, uint32_t lane, uint32_t *s, uint32_t stride) const
    {
        stage_words(s, reinterpret_cast<const uint32_t *>(rank), i0, n, lane);
        const uint32_t base = i0 & ~3u, nw = ((i0 & 3u) + n + 3u) >> 2;
        for (uint32_t c = lane; c < nw; c += 32) cp_async4(s + stride + c, wl_curr + base + 4u * c);
    }
    __device__ __forceinline__ RowPre unstage(uint32_t, const uint32_t *s, uint32_t j, uint32_t stride) const
    {
        return RowPre{__uint_as_float(s[j]), (s[stride + (j >> 2)] >> (8u * (j & 3u))) & 0xffu};
    }
    __device__ __forceinline__ void finish(uint32_t r, float sum, const RowPre &pre, double &err, uint32_t &act)
    {
        if (!pre.on) return;
        float nr = __fadd_rn(base, __fmul_rn(damp, sum));
        float pr = pre.rank;
        float e = fabsf(__fsub_rn(nr, pr));
        err += (double)e;
        if (e >= eps_f)
        {
            rank[r] = nr;
            for (uint32_t j = out_off[r]; j < out_off[r + 1]; j++) wl_next[out_adj[j]] = 1;
            act++;
        }
    }
    __device__ __forceinline__ void warp_end(double err, uint32_t act) { warp_reduce(err, act); }
};

__global__ void __launch_bounds__(GG_TILE_NT) k_dd_pull(const uint32_t *__restrict__ off, const uint32_t *__restrict__ adj,
                                                        const uint2 *__restrict__ coord, uint32_t ntiles, float *g_acc,
                                                        DdPullOp op)
{
    if (op.skip()) return;
    warp_pull<GG_TILE_IPT, GG_TILE_WARPS>(off, adj, op.V, coord, ntiles, g_acc, op);
}

__global__ void __launch_bounds__(256) k_dd_pull_fixup(const uint32_t *__restrict__ off, const uint2 *__restrict__ coord,
                                                       uint32_t ntiles, float *g_acc, DdPullOp op)
{
    if (op.skip()) return;
    warp_pull_fixup(off, op.V, coord, ntiles, GG_TILE_ITEMS, g_acc, op);
}

/* data-driven push (mode 7) and pull-push (mode 8): one warp per worklist
 * vertex; residuals move with atomics, as the reference's OpenMP loop does */
__global__ void k_dd_residual_init(const uint32_t *__restrict__ in_off, const uint32_t *__restrict__ in_adj,
                                   const uint32_t *__restrict__ outdeg, float *resid, uint8_t *wl, uint32_t V, float damp)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t v = warp; v < V; v += nwarps)
    {
        float r = 0.0f;
        for (uint32_t j = in_off[v] + lane; j < in_off[v + 1]; j += 32)
        {
            uint32_t du = outdeg[in_adj[j]];
            if (du) r += __fdiv_rn(1.0f, __uint2float_rn(du));
        }
        r = warp_sum(r);
        if (lane == 0)
        {
            resid[v] = __fmul_rn(__fmul_rn(__fsub_rn(1.0f, damp), damp), r);
            wl[v] = 1;
        }
    }
}

__global__ void k_dd_push(PrCommon c, int pullpush, const uint32_t *__restrict__ in_off, const uint32_t *__restrict__ in_adj,
                          const uint32_t *__restrict__ out_off, const uint32_t *__restrict__ out_adj, float *resid,
                          const uint8_t *wl_curr, uint8_t *wl_next)
{
    if (c.skip()) return;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    double err = 0.0;
    uint32_t act = 0;
    for (uint32_t v = warp; v < c.V; v += nwarps)
    {
        if (!wl_curr[v]) continue;
        float old_pr = c.rank[v];
        float new_pr;
        float rv;
        if (!pullpush)
        {
            rv = 0.0f;
            if (lane == 0) rv = atomicExch(&resid[v], 0.0f);
            rv = __shfl_sync(0xffffffffu, rv, 0);
            new_pr = __fadd_rn(rv, old_pr);
        }
        else
        {
            float in_pr = 0.0f;
            for (uint32_t j = in_off[v] + lane; j < in_off[v + 1]; j += 32)
            {
                uint32_t u = in_adj[j];
                in_pr += __fdiv_rn(c.rank[u], __uint2float_rn(c.outdeg[u]));
            }
            in_pr = __shfl_sync(0xffffffffu, warp_sum(in_pr), 0);
            new_pr = __fadd_rn(c.base, __fmul_rn(c.damp, in_pr));
            rv = 0.0f;
            if (lane == 0) rv = atomicExch(&resid[v], 0.0f);
            rv = __shfl_sync(0xffffffffu, rv, 0);
        }
        if (lane == 0)
        {
            float fv = __uint2float_rn(c.V);
            err += fabs((double)__fsub_rn(__fdiv_rn(new_pr, fv), __fdiv_rn(old_pr, fv)));
            c.rank[v] = new_pr;
        }
        uint32_t deg = c.outdeg[v];
        float delta = __fmul_rn(c.damp, __fdiv_rn(rv, __uint2float_rn(deg)));
        for (uint32_t j = out_off[v] + lane; j < out_off[v + 1]; j += 32)
        {
            uint32_t u = out_adj[j];
            float prev = atomicAdd(&resid[u], delta);
            if (fabsf(__fadd_rn(prev, delta)) >= c.eps_f && prev <= c.eps_fl)
            {
                act++;
                if (pullpush) atomicAdd(&resid[u], delta);
                wl_next[u] = 1;
            }
        }
    }
    block_sum2<256>(err, act);
    if (threadIdx.x == 0) c.reduce(err, act);
}

__global__ void k_clear_bytes(uint8_t *p, uint32_t n, IterRec *rec, uint32_t it)
{
    if (it > 0 && rec[it - 1].active == 0u) return;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = 0;
}

/* ---- host driver ------------------------------------------------------------------ */

struct Run
{
    gg_graph *g;
    cudaStream_t s;
    const gg_pr_params *p;
    float eps_f = 0.0f, eps_fl = 0.0f;
    uint32_t launches = 0;
    uint32_t gather_launches = 0;
    float gather_ms = 0.0f;
    std::vector<cudaEvent_t> evs;
};

int grid_v(uint32_t V) { int b = (int)((V + 255) / 256); int cap = gg_sm_count() * 8; return b < 1 ? 1 : (b > cap ? cap : b); }
int fixup_grid(uint32_t ntiles) { return grid_v(ntiles); }

gg_status timed_begin(Run &R)
{
    if (!R.p->profile) return GG_OK;
    cudaEvent_t e;
    GG_CHECK(gg_event_at(R.g, (uint32_t)R.evs.size(), &e));
    GG_CUDA(cudaEventRecord(e, R.s));
    R.evs.push_back(e);
    return GG_OK;
}
gg_status timed_end(Run &R) { return timed_begin(R); }

template <int K>
gg_status run_pull(Run &R, IterRec *rec, float *rank, uint32_t iters, float base, float init)
{
    typedef typename Fmt<K>::CT CT;
    typedef typename Fmt<K>::Acc Acc;
    gg_graph *g = R.g;
    const uint32_t V = g->V;
    gg_tiles *t;
    GG_CHECK(gg_tiles_get(g, 1, R.s, &t));
    void *c0, *c1, *cf = nullptr;
    GG_CHECK(gg_work(g, 2, ((size_t)V + 16) * sizeof(CT), &c0));
    GG_CHECK(gg_work(g, 3, ((size_t)V + 16) * sizeof(CT), &c1));
    if (Fmt<K>::quant) GG_CHECK(gg_work(g, 4, ((size_t)V + 16) * sizeof(float), &cf));
    CT *cb[2] = {(CT *)c0, (CT *)c1};

    k_pr_init<K><<<grid_v(V), 256, 0, R.s>>>(rank, g->out_deg, V, init, Fmt<K>::quant ? nullptr : cb[0],
                                               (float *)cf, rec);
    R.launches++;
    for (uint32_t it = 0; it < iters; it++)
    {
        if constexpr (Fmt<K>::quant)
        {
            k_quantize<CT><<<grid_v(V), 256, 0, R.s>>>((const float *)cf, cb[0], V, Fmt<K>::bits, 0, rec, it, nullptr);
            R.launches++;
        }
        PullOp<K> op;
        op.rank = rank; op.outdeg = g->out_deg; op.V = V; op.base = base; op.damp = R.p->damp;
        op.eps_f = R.eps_f; op.eps_fl = R.eps_fl; op.rec = rec; op.it = it;
        op.cin = Fmt<K>::quant ? cb[0] : cb[it & 1];
        op.cout = cb[(it + 1) & 1];
        op.cf = (float *)cf;
        GG_CHECK(timed_begin(R));
        k_pr_pull<K><<<gg_persistent_grid((const void *)k_pr_pull<K>, t->ntiles, GG_PULL_CTAS_PER_SM), GG_TILE_NT, 0, R.s>>>(
            g->in_off, g->in_adj, t->coord, t->ntiles, (Acc *)t->acc, op);
        k_pr_pull_fixup<K><<<fixup_grid(t->ntiles), 256, 0, R.s>>>(g->in_off, t->coord, t->ntiles, (Acc *)t->acc, op);
        GG_CHECK(timed_end(R));
        R.launches += 2;
        R.gather_launches++;
    }
    GG_CUDA(cudaGetLastError());
    return GG_OK;
}

template <int K>
gg_status run_push(Run &R, IterRec *rec, float *rank, uint32_t iters, float base, float init)
{
    /* K is K_F32/K_BF16/K_F16 (float scatter), K_FX64, or K_Q8Z */
    typedef typename Fmt<(K == K_Q8Z ? K_Q8 : K)>::CT CT;
    gg_graph *g = R.g;
    const uint32_t V = g->V;
    gg_tiles *t;
    GG_CHECK(gg_tiles_get(g, 0, R.s, &t));
    void *c0, *nx, *cf = nullptr, *zeros = nullptr;
    GG_CHECK(gg_work(g, 2, ((size_t)V + 16) * sizeof(CT), &c0));
    GG_CHECK(gg_work(g, 5, ((size_t)V + 16) * 8, &nx));
    GG_CUDA(cudaMemsetAsync(nx, 0, ((size_t)V + 16) * 8, R.s));
    if (K == K_Q8Z)
    {
        GG_CHECK(gg_work(g, 4, ((size_t)V + 16) * sizeof(float), &cf));
        GG_CHECK(gg_work(g, 6, ((size_t)iters + 2) * 4, &zeros));
    }
    constexpr int KI = (K == K_Q8Z ? K_Q8 : K);
    if constexpr (K == K_Q8Z)
        k_pr_init<K_Q8><<<grid_v(V), 256, 0, R.s>>>(rank, g->out_deg, V, init, nullptr, (float *)cf, rec);
    else
        k_pr_init<K><<<grid_v(V), 256, 0, R.s>>>(rank, g->out_deg, V, init, (CT *)c0, nullptr, rec);
    R.launches++;
    for (uint32_t it = 0; it < iters; it++)
    {
        GG_CHECK(timed_begin(R));
        if constexpr (K == K_Q8Z)
        {
            k_quantize<uint8_t><<<grid_v(V), 256, 0, R.s>>>((const float *)cf, (uint8_t *)c0, V, 8, 1, rec, it,
                                                           (uint32_t *)zeros);
            k_pr_push_q<<<gg_persistent_grid((const void *)k_pr_push_q, t->ntiles), GG_TILE_NT, 0, R.s>>>(
                g->out_off, g->out_adj, t->coord, t->ntiles, V, (const uint8_t *)c0,
                                                           (const uint32_t *)zeros, (float *)nx, rec, it);
            R.launches += 2;
        }
        else if constexpr (K == K_FX64)
        {
            k_pr_push_fx64<<<gg_persistent_grid((const void *)k_pr_push_fx64, t->ntiles), GG_TILE_NT, 0, R.s>>>(
                g->out_off, g->out_adj, t->coord, t->ntiles, V,
                                                              (const unsigned long long *)c0, (unsigned long long *)nx, rec, it);
            R.launches++;
        }
        else
        {
            k_pr_push_f<K><<<gg_persistent_grid((const void *)k_pr_push_f<K>, t->ntiles), GG_TILE_NT, 0, R.s>>>(
                g->out_off, g->out_adj, t->coord, t->ntiles, V, (const CT *)c0,
                                                              (float *)nx, rec, it);
            R.launches++;
        }
        GG_CHECK(timed_end(R));
        R.gather_launches++;
        PrCommon c;
        c.rank = rank; c.outdeg = g->out_deg; c.V = V; c.base = base; c.damp = R.p->damp;
        c.eps_f = R.eps_f; c.eps_fl = R.eps_fl; c.rec = rec; c.it = it;
        if constexpr (K == K_FX64)
            k_pr_push_update<K_FX64><<<grid_v(V), 256, 0, R.s>>>(c, (unsigned long long *)nx, (unsigned long long *)c0, nullptr);
        else if constexpr (K == K_Q8Z)
            k_pr_push_update<K_Q8Z><<<grid_v(V), 256, 0, R.s>>>(c, (float *)nx, nullptr, (float *)cf);
        else
            k_pr_push_update<K><<<grid_v(V), 256, 0, R.s>>>(c, (float *)nx, (CT *)c0, nullptr);
        R.launches++;
    }
    (void)KI;
    GG_CUDA(cudaGetLastError());
    return GG_OK;
}

gg_status run_dd(Run &R, int mode, IterRec *rec, float *rank, uint32_t iters, float base, float init)
{
    gg_graph *g = R.g;
    const uint32_t V = g->V;
    if (!g->in_off || !g->out_off) return gg_fail(GG_ERR_INVALID, "data-driven PageRank needs GG_MAP_IN|GG_MAP_OUT");
    void *cf, *wa, *wb, *resid = nullptr;
    GG_CHECK(gg_work(g, 4, ((size_t)V + 16) * 4, &cf));
    GG_CHECK(gg_work(g, 7, (size_t)V + 16, &wa));
    GG_CHECK(gg_work(g, 8, (size_t)V + 16, &wb));
    GG_CUDA(cudaMemsetAsync(wa, 0, (size_t)V + 16, R.s));
    GG_CUDA(cudaMemsetAsync(wb, 0, (size_t)V + 16, R.s));
    k_pr_init<K_F32><<<grid_v(V), 256, 0, R.s>>>(rank, g->out_deg, V, init, nullptr, nullptr, rec);
    R.launches++;
    uint8_t *wl[2] = {(uint8_t *)wa, (uint8_t *)wb};
    if (mode == GG_PR_DD_PULL)
    {
        GG_CUDA(cudaMemsetAsync(wa, 1, V, R.s));
        gg_tiles *t;
        GG_CHECK(gg_tiles_get(g, 1, R.s, &t));
        for (uint32_t it = 0; it < iters; it++)
        {
            k_dd_contrib<<<grid_v(V), 256, 0, R.s>>>(rank, g->out_deg, (float *)cf, V, rec, it);
            DdPullOp op;
            op.rank = rank; op.outdeg = g->out_deg; op.V = V; op.base = base; op.damp = R.p->damp;
            op.eps_f = R.eps_f; op.eps_fl = R.eps_fl; op.rec = rec; op.it = it;
            op.cf = (const float *)cf; op.wl_curr = wl[it & 1]; op.wl_next = wl[(it + 1) & 1];
            op.out_off = g->out_off; op.out_adj = g->out_adj;
            GG_CHECK(timed_begin(R));
            k_dd_pull<<<gg_persistent_grid((const void *)k_dd_pull, t->ntiles, GG_PULL_CTAS_PER_SM), GG_TILE_NT, 0, R.s>>>(
                g->in_off, g->in_adj, t->coord, t->ntiles, (float *)t->acc, op);
            k_dd_pull_fixup<<<fixup_grid(t->ntiles), 256, 0, R.s>>>(g->in_off, t->coord, t->ntiles, (float *)t->acc, op);
            GG_CHECK(timed_end(R));
            k_clear_bytes<<<grid_v(V), 256, 0, R.s>>>(wl[it & 1], V, rec, it);
            R.launches += 4;
            R.gather_launches++;
        }
    }
    else
    {
        GG_CHECK(gg_work(g, 9, ((size_t)V + 16) * 4, &resid));
        k_dd_residual_init<<<gg_sm_count() * 8, 256, 0, R.s>>>(g->in_off, g->in_adj, g->out_deg, (float *)resid,
                                                              wl[0], V, R.p->damp);
        R.launches++;
        for (uint32_t it = 0; it < iters; it++)
        {
            PrCommon c;
            c.rank = rank; c.outdeg = g->out_deg; c.V = V; c.base = base; c.damp = R.p->damp;
            c.eps_f = R.eps_f; c.eps_fl = R.eps_fl; c.rec = rec; c.it = it;
            GG_CHECK(timed_begin(R));
            k_dd_push<<<gg_sm_count() * 8, 256, 0, R.s>>>(c, mode == GG_PR_DD_PULLPUSH, g->in_off, g->in_adj, g->out_off,
                                                          g->out_adj, (float *)resid, wl[it & 1], wl[(it + 1) & 1]);
            GG_CHECK(timed_end(R));
            k_clear_bytes<<<grid_v(V), 256, 0, R.s>>>(wl[it & 1], V, rec, it);
            R.launches += 2;
            R.gather_launches++;
        }
    }
    GG_CUDA(cudaGetLastError());
    return GG_OK;
}

} // namespace

extern "C" gg_status gg_pagerank(gg_graph *g, const gg_pr_params *p, float *ranks, gg_pr_result *r, void *stream)
{
    if (!g || !p) return gg_fail(GG_ERR_INVALID, "NULL argument");
    if (p->mode > 13) return gg_fail(GG_ERR_INVALID, "unknown PageRank mode");
    if (p->storage > 2) return gg_fail(GG_ERR_INVALID, "unknown storage");
    const int pull = !(p->mode == GG_PR_PUSH || p->mode == GG_PR_PUSH_FX64 || p->mode == GG_PR_PUSH_Q ||
                       p->mode == GG_PR_DD_PUSH || p->mode == GG_PR_DD_PULLPUSH);
    if (pull && !g->in_off) return gg_fail(GG_ERR_INVALID, "pull PageRank needs GG_MAP_IN");
    if (!pull && !g->out_off) return gg_fail(GG_ERR_INVALID, "push PageRank needs GG_MAP_OUT");
    if (!g->out_deg) return gg_fail(GG_ERR_INVALID, "mapping has no out-degrees");

    Run R;
    R.g = g;
    R.s = gg_stream(g, stream);
    R.p = p;
    R.eps_f = gg_float_ceil(p->epsilon);
    R.eps_fl = gg_float_floor(p->epsilon);
    const uint32_t V = g->V, iters = p->max_iterations;
    gg_pr_result res;
    memset(&res, 0, sizeof(res));

    void *rank_v, *rec_v, *sum_v;
    GG_CHECK(gg_work(g, 0, ((size_t)V + 16) * 4, &rank_v));
    GG_CHECK(gg_work(g, 1, ((size_t)iters + 2) * sizeof(IterRec), &rec_v));
    GG_CHECK(gg_work(g, 10, 64, &sum_v));
    IterRec *rec = (IterRec *)rec_v;
    float *rank = (float *)rank_v;
    GG_CUDA(cudaMemsetAsync(rec, 0, ((size_t)iters + 2) * sizeof(IterRec), R.s));
    GG_CUDA(cudaMemsetAsync(sum_v, 0, 64, R.s));

    const float damp = p->damp;
    const float base_pr = 1.0f - damp;
    const float base = p->init_one_over_n ? base_pr / (float)V : base_pr;
    const float init = p->init_one_over_n ? 1.0f / (float)V : base_pr;

    if (V > 0)
    {
        gg_status st = GG_OK;
        switch (p->mode)
        {
        case GG_PR_PULL:
            st = p->storage == GG_STORE_BF16 ? run_pull<K_BF16>(R, rec, rank, iters, base, init)
                 : p->storage == GG_STORE_F16 ? run_pull<K_F16>(R, rec, rank, iters, base, init)
                                              : run_pull<K_F32>(R, rec, rank, iters, base, init);
            break;
        case GG_PR_PULL_FX64: st = run_pull<K_FX64>(R, rec, rank, iters, base, init); break;
        case GG_PR_PULL_FX32: st = run_pull<K_FX32>(R, rec, rank, iters, base, init); break;
        case GG_PR_PULL_FX16: st = run_pull<K_FX16>(R, rec, rank, iters, base, init); break;
        case GG_PR_PULL_FX8: st = run_pull<K_FX8>(R, rec, rank, iters, base, init); break;
        case GG_PR_PULL_Q32: st = run_pull<K_Q32>(R, rec, rank, iters, base, init); break;
        case GG_PR_PULL_Q16: st = run_pull<K_Q16>(R, rec, rank, iters, base, init); break;
        case GG_PR_PULL_Q8: st = run_pull<K_Q8>(R, rec, rank, iters, base, init); break;
        case GG_PR_PUSH:
            st = p->storage == GG_STORE_BF16 ? run_push<K_BF16>(R, rec, rank, iters, base, init)
                 : p->storage == GG_STORE_F16 ? run_push<K_F16>(R, rec, rank, iters, base, init)
                                              : run_push<K_F32>(R, rec, rank, iters, base, init);
            break;
        case GG_PR_PUSH_FX64: st = run_push<K_FX64>(R, rec, rank, iters, base, init); break;
        case GG_PR_PUSH_Q: st = run_push<K_Q8Z>(R, rec, rank, iters, base, init); break;
        default: st = run_dd(R, (int)p->mode, rec, rank, iters, base, init); break;
        }
        if (st != GG_OK) return st;
        k_pr_finalize<<<grid_v(V), 256, 0, R.s>>>(rank, V, p->init_one_over_n ? 0 : 1, (double *)sum_v);
        R.launches++;
        GG_CUDA(cudaGetLastError());
    }

    std::vector<IterRec> h(iters + 2);
    double sum = 0.0;
    GG_CUDA(cudaMemcpyAsync(h.data(), rec, ((size_t)iters + 2) * sizeof(IterRec), cudaMemcpyDeviceToHost, R.s));
    GG_CUDA(cudaMemcpyAsync(&sum, sum_v, sizeof(double), cudaMemcpyDeviceToHost, R.s));
    if (ranks && V) GG_CUDA(cudaMemcpyAsync(ranks, rank, (size_t)V * 4, cudaMemcpyDeviceToHost, R.s));
    GG_CHECK(gg_wait(R.s));

    /* reference loop convention: iterations = index of the breaking
     * iteration, or max when the loop ran out (pageRank.c:1021-1075) */
    uint32_t k = 0;
    for (; k < iters; k++)
        if (h[k].active == 0u) break;
    res.iterations = k;
    const uint32_t last = k < iters ? k : (iters ? iters - 1 : 0);
    res.active = iters ? h[last].active : 0;
    /* the kernels sum |delta|; the data-driven push variants add terms
     * already divided by V (pageRank.c:3049) */
    const bool pre_scaled = p->mode == GG_PR_DD_PUSH || p->mode == GG_PR_DD_PULLPUSH;
    res.error_total = iters ? (pre_scaled ? h[last].err : h[last].err / (double)V) : 0.0;
    res.rank_sum = sum;
    res.launches = R.launches;
    res.gather_launches = R.gather_launches;
    if (p->profile)
    {
        float ms = 0.0f;
        for (size_t i = 0; i + 1 < R.evs.size(); i += 2) ms += gg_event_ms(R.evs[i], R.evs[i + 1]);
        res.gather_ms = ms;
    }
    g->last_ranks = rank;
    if (r) *r = res;
    return GG_OK;
}

extern "C" const float *gg_pagerank_device_ranks(const gg_graph *g) { return g ? g->last_ranks : nullptr; }
