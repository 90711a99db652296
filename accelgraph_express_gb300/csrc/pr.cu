/*
 * PageRank on CSR, all fourteen variants of the reference's dispatcher
 * (02_capi_graph/src/algorithms/capi/pageRank.c:874-939), on one GPU.
 *
 * Topology-driven pull (modes 0, 2, 4, 9-13): per iteration the merge-path
 * tile gather over the CSC writes every vertex's sum, then one vertex pass
 * runs the reference's update (pageRank.c:1055-1069) fused with the next
 * iteration's contribution pass (pageRank.c:1026-1033):
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
 * Storage: contributions in FP32, or in the fixed-point / quantised integer
 * formats summed exactly in 64 bits, or 16-bit BF16 / FP16 with an FP32
 * correction pass: the gathered 16-bit values are per-iteration deltas of
 * each vertex's contribution, and the vertex pass keeps the FP32 running
 * sums and the FP32 value of everything stored so far, so every iteration
 * stores the rounding of (contribution - stored so far) and no rounding
 * error accumulates (k_pr_update_delta).
 *
 * From 1M vertices the FP pull gather reads the contributions of the
 * vertices with the most out-edges from a shared-memory table
 * (k_pr_pull_hot, table built by hot.cu).  With GG_PR_CUDA_GRAPH the whole
 * call is captured once into a CUDA graph kept on the mapping and relaunched
 * by later calls with the same parameters.
 */
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
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
    uint32_t maxbits;  /* max contribution (float bits) for the quantised modes; max |delta| for BF16/FP16 */
    float qinv;        /* BF16/FP16: 1 / the scale this iteration's stored deltas were written with */
    uint32_t pad;
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
    __device__ __forceinline__ void reduce(double err, uint32_t act) const
    {
        if (err != 0.0) atomicAdd(&rec[it].err, err);
        if (act) atomicAdd(&rec[it].active, act);
    }
};

/* ---- pull: gather, then vertex update ---------------------------------------------- */

/* the edge term of the pull gather: the in-neighbour's stored contribution */
template <int K>
struct PrGather
{
    typedef typename Fmt<K>::Acc Acc;
    typedef typename Fmt<K>::CT Raw;
    const Raw *cin;
    __device__ __forceinline__ Raw load(uint32_t, uint32_t u) const { return ldg_val(cin + u); }
    __device__ __forceinline__ Acc value(const Raw &r) const { return decode<K>(r); }
};

/* the gather with the hot-vertex table: flagged ids read the table */
template <int K>
struct PrGatherHot
{
    typedef typename Fmt<K>::Acc Acc;
    typedef typename Fmt<K>::CT Raw;
    const Raw *cin;
    const Raw *s_hot;
    __device__ __forceinline__ Raw load(uint32_t, uint32_t u) const
    {
        if (u & GG_HOT_FLAG) return s_hot[u & ~GG_HOT_FLAG];
        return ldg_val(cin + u);
    }
    __device__ __forceinline__ Acc value(const Raw &r) const { return decode<K>(r); }
};

template <int K>
__host__ __device__ constexpr uint32_t hot_entries()
{
    return GG_HOT_TABLE_BYTES / sizeof(typename Fmt<K>::CT) < GG_HOT_ENTRIES
               ? (uint32_t)(GG_HOT_TABLE_BYTES / sizeof(typename Fmt<K>::CT))
               : GG_HOT_ENTRIES;
}
template <int K>
__host__ __device__ constexpr size_t hot_stage_bytes(uint32_t warps)
{
    return (size_t)warps * PullStage<GG_HOT_IPT, typename Fmt<K>::Acc>::BYTES;
}
template <int K>
__host__ __device__ constexpr size_t hot_smem_bytes(uint32_t warps)
{
    return hot_stage_bytes<K>(warps) + ((size_t)hot_entries<K>() * sizeof(typename Fmt<K>::CT) + 15) / 16 * 16;
}

/* one CTA per SM (up to GG_HOT_WARPS warps, the tuned count): the CTA fills
 * the table with the hot vertices' stored contributions, then its warps run
 * the engine */
template <int K>
__global__ void __launch_bounds__(GG_HOT_WARPS * 32, 1)
    k_pr_pull_hot(const uint32_t *__restrict__ off, const uint32_t *__restrict__ hot_adj,
                  const uint2 *__restrict__ coord, uint32_t ntiles, uint32_t V, typename Fmt<K>::Acc *sums,
                  const typename Fmt<K>::CT *__restrict__ cin, const uint32_t *__restrict__ hot_list, uint32_t hot_n,
                  const IterRec *rec, uint32_t it)
{
    typedef typename Fmt<K>::CT CT;
    extern __shared__ __align__(16) unsigned char gg_dyn[];
    pdl_wait();
    if (it > 0 && rec[it - 1].active == 0u) return;
    CT *s_hot = reinterpret_cast<CT *>(gg_dyn + hot_stage_bytes<K>(blockDim.x >> 5));
    for (uint32_t i = threadIdx.x; i < hot_n; i += blockDim.x) s_hot[i] = cin[hot_list[i]];
    __syncthreads();
    warp_pull_sums_dyn<GG_HOT_IPT>(gg_dyn, off, hot_adj, V, coord, ntiles, sums, PrGatherHot<K>{cin, s_hot});
    pdl_trigger();
}

/* grid of k_pr_pull_hot<K> with `warps` warps: one CTA per SM, the
 * carve-out sized to its shared memory (the rest of the array stays L1) */
template <int K>
int hot_grid(uint32_t ntiles, uint32_t warps)
{
    static int ok = -1;
    static uint32_t applied = 0;
    int dev = 0, smem_sm = 0;
    if (ok < 0)
    {
        const size_t most = hot_smem_bytes<K>(GG_HOT_WARPS);
        cudaError_t e = cudaFuncSetAttribute(k_pr_pull_hot<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)most);
        ok = e == cudaSuccess ? 1 : 0;
        if (!ok) cudaGetLastError();
    }
    if (!ok) return 0;
    if (applied != warps)
    {
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
        if (smem_sm > 0)
        {
            const int pct = (int)ceil(100.0 * (double)(hot_smem_bytes<K>(warps) + 1024) / (double)smem_sm);
            if (cudaFuncSetAttribute(k_pr_pull_hot<K>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     pct > 100 ? 100 : pct) == cudaSuccess)
                applied = warps;
            else
                cudaGetLastError();
        }
    }
    const uint32_t need = (ntiles + warps - 1) / warps;
    const uint32_t cap = (uint32_t)gg_sm_count();
    return (int)(need < cap ? (need ? need : 1) : cap);
}

template <int K>
__global__ void __launch_bounds__(GG_TILE_NT) k_pr_pull(const uint32_t *__restrict__ off,
                                                        const uint32_t *__restrict__ adj, const uint2 *__restrict__ coord,
                                                        uint32_t ntiles, uint32_t V, typename Fmt<K>::Acc *sums,
                                                        PrGather<K> op, const IterRec *rec, uint32_t it)
{
    pdl_wait();
    if (it > 0 && rec[it - 1].active == 0u) return;
    warp_pull_sums<GG_TILE_IPT, GG_TILE_WARPS>(off, adj, V, coord, ntiles, sums, op);
    pdl_trigger();
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
    pdl_wait();
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

/* final normalisation of a batch of graphs (vertex ranges voff[g] ..
 * voff[g+1]): each vertex is divided by its own graph's vertex count */
__global__ void k_pr_finalize_seg(float *__restrict__ rank, uint32_t V, const uint32_t *__restrict__ voff,
                                  uint32_t ngraphs, double *sum)
{
    double s = 0.0;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
    {
        /* graph of v: the last g with voff[g] <= v */
        uint32_t lo = 0, hi = ngraphs - 1;
        while (lo < hi)
        {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (voff[mid] <= v)
                lo = mid;
            else
                hi = mid - 1;
        }
        const float r = __fdiv_rn(rank[v], __uint2float_rn(voff[lo + 1] - voff[lo]));
        rank[v] = r;
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

/* vertex update from the gathered (pull) or scattered (push) sums
 * (pageRank.c:1055-1069 and :2067-2081), fused with the next iteration's
 * contribution pass (pageRank.c:1026-1033); clears sums for the next launch */
template <int K>
__global__ void k_pr_update(PrCommon c, typename Fmt<K>::Acc *sums, typename Fmt<K>::CT *cout, float *cf)
{
    pdl_wait();
    if (c.skip()) return;
    double err = 0.0;
    uint32_t act = 0, tmax = 0;
    float qscale = 0.0f;
    if constexpr (Fmt<K>::quant && K != K_Q8Z) qscale = quant_scale(c.rec[c.it].maxbits, Fmt<K>::bits);
    typename Fmt<K>::Acc *__restrict__ sv = sums;
    float *__restrict__ rank = c.rank;
    const uint32_t *__restrict__ outdeg = c.outdeg;
    uint32_t v0 = 0;
    if constexpr (K == K_F32)
    {
        /* FP32: two adjacent vertices per step in 8-byte loads and stores
         * (more loads in flight; every array is a whole allocation), the
         * same arithmetic per vertex as the loop below */
        const uint32_t P = c.V >> 1;
        for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x)
        {
            const float2 s = reinterpret_cast<const float2 *>(sv)[p];
            const float2 pr = reinterpret_cast<const float2 *>(rank)[p];
            const uint2 d = reinterpret_cast<const uint2 *>(outdeg)[p];
            if (s.x != 0.0f || s.y != 0.0f) reinterpret_cast<float2 *>(sv)[p] = make_float2(0.0f, 0.0f);
            const float2 nr = make_float2(next_rank<K>(c.base, c.damp, s.x, 0.0f), next_rank<K>(c.base, c.damp, s.y, 0.0f));
            reinterpret_cast<float2 *>(rank)[p] = nr;
            const float e0 = fabsf(__fsub_rn(nr.x, pr.x)), e1 = fabsf(__fsub_rn(nr.y, pr.y));
            err += (double)e0;
            err += (double)e1;
            act += (e0 >= c.eps_f) + (e1 >= c.eps_f);
            reinterpret_cast<float2 *>(cout)[p] = make_float2(encode<K>(contrib_of(nr.x, d.x), d.x),
                                                              encode<K>(contrib_of(nr.y, d.y), d.y));
        }
        v0 = P * 2;
    }
    for (uint32_t v = v0 + blockIdx.x * blockDim.x + threadIdx.x; v < c.V; v += gridDim.x * blockDim.x)
    {
        const typename Fmt<K>::Acc s = sv[v];
        const float pr = rank[v];
        const uint32_t d = outdeg[v];
        float nr;
        if constexpr (K == K_Q8Z)
            nr = __fadd_rn(c.base, __fmul_rn(c.damp, (float)s));
        else
            nr = next_rank<K>(c.base, c.damp, s, qscale);
        clear_after_read(&sv[v], s);
        rank[v] = nr;
        /* pageRank.c:1057-1067: |rank' - rank| is a float difference, exact
         * in FP64; the FP64 sum of the differences is divided by V once on
         * the host (the reference divides each term), and `error >= epsilon`
         * is the same test as e >= eps_f in FP32, so no FP64 division or
         * compare runs per vertex (FP64 is a small fraction of the FP32 rate
         * here) */
        const float e = fabsf(__fsub_rn(nr, pr));
        err += (double)e;
        if (e >= c.eps_f) act++;
        float ctb = contrib_of(nr, d);
        if constexpr (Fmt<K>::quant)
        {
            cf[v] = ctb;
            tmax = max(tmax, __float_as_uint(ctb));
        }
        else
            cout[v] = encode<K>(ctb, d);
    }
    if constexpr (Fmt<K>::quant) block_max_bits<256>(tmax, &c.rec[c.it + 1].maxbits);
    block_sum2<256>(err, act);
    if (threadIdx.x == 0) c.reduce(err, act);
    pdl_trigger();
}

/* ---- BF16 / FP16 storage with the FP32 correction pass ------------------------- */

/* FP16 deltas are stored multiplied by a power of two chosen from the
 * largest |delta| of the previous iteration, which lands at 2^13 .. 2^14
 * (deltas may grow 4x before FP16's 65504 saturates; a saturated or
 * underflowed part stays in the next delta).  Returns the exponent. */
__device__ __forceinline__ int f16_scale_exp(uint32_t maxbits)
{
    const int be = (int)((maxbits >> 23) & 0xffu);
    if (be == 0) return 0; /* zero (or subnormal) deltas: scale 1 */
    int k = 13 - (be - 127);
    return k < -120 ? -120 : (k > 120 ? 120 : k);
}
__device__ __forceinline__ float pow2f(int k) { return __uint_as_float((uint32_t)(127 + k) << 23); }

/* store delta d (FP32) in format K with scale 2^k; returns the value the
 * gather will see, unscaled (exact: a power-of-two product) */
template <int K>
__device__ __forceinline__ float store_delta(float d, int k, typename Fmt<K>::CT *q)
{
    if constexpr (K == K_BF16)
    {
        const __nv_bfloat16 b = __float2bfloat16_rn(d);
        *q = b;
        return __bfloat162float(b);
    }
    else
    {
        float x = __fmul_rn(d, pow2f(k));
        x = fminf(fmaxf(x, -65504.0f), 65504.0f);
        const __half h = __float2half_rn(x);
        *q = h;
        return __fmul_rn(__half2float(h), pow2f(-k));
    }
}

/* initial state: rank = init, nothing stored yet, so the first delta is the
 * whole first contribution; FP16's first scale comes from `init`, the
 * largest contribution there is (out-degrees are >= 1) */
template <int K>
__global__ void k_pr_init_delta(float *__restrict__ rank, const uint32_t *__restrict__ outdeg, uint32_t V, float init,
                                typename Fmt<K>::CT *qout, float *__restrict__ S, float *__restrict__ chat, IterRec *rec)
{
    const int k = K == K_F16 ? f16_scale_exp(__float_as_uint(init)) : 0;
    uint32_t tmax = 0;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
    {
        rank[v] = init;
        const float c = contrib_of(init, outdeg[v]);
        S[v] = 0.0f;
        chat[v] = store_delta<K>(c, k, &qout[v]);
        tmax = max(tmax, __float_as_uint(c));
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) rec[0].qinv = pow2f(-k);
    block_max_bits<256>(tmax, &rec[0].maxbits);
}

/* The FP32 correction pass: the vertex update (pageRank.c:1055-1069, fused
 * with the contribution pass :1026-1033) for 16-bit storage.  dsum[v] is
 * the gathered (pull) or scattered (push) sum of the in-neighbours' stored
 * deltas; S[v] is the FP32 sum of everything gathered so far (the sum of
 * the in-neighbours' stored contributions), chat[v] the FP32 value of
 * everything v has stored so far.  rank' = 0.15 + 0.85 * S, the next stored
 * delta is round16(contrib' - chat): what one iteration's rounding lost is
 * sent in the next, so the ranks carry only the rounding of the last delta,
 * which shrinks as the iteration converges. */
/* one vertex of the correction pass from its loaded values: returns the new
 * running sum in s, the rank in nr, the stored-so-far value in ch and the
 * stored 16-bit delta in q */
template <int K>
struct DeltaStep
{
    typedef typename Fmt<K>::CT CT;
    float base, damp, init, in_inv, eps_f;
    int k;
    bool first;
    double err;
    uint32_t act, tmax;
    __device__ __forceinline__ void operator()(float ds, float &s, float &ch, uint32_t deg, float &nr, CT &q)
    {
        const float s_old = s;
        s = __fadd_rn(s_old, __fmul_rn(ds, in_inv));
        /* the rank the previous pass wrote, recomputed from its sum (the same
         * two roundings), so the rank array is only written: a store to a
         * sector whose read is still in flight stalls */
        const float pr = first ? init : __fadd_rn(base, __fmul_rn(damp, s_old));
        nr = __fadd_rn(base, __fmul_rn(damp, s));
        const float e = fabsf(__fsub_rn(nr, pr));
        err += (double)e;
        if (e >= eps_f) act++;
        const float d = __fsub_rn(contrib_of(nr, deg), ch);
        ch = __fadd_rn(ch, store_delta<K>(d, k, &q));
        tmax = max(tmax, __float_as_uint(fabsf(d)));
    }
};

template <class CT> struct Pair16;
template <> struct Pair16<__nv_bfloat16> { typedef __nv_bfloat162 T; static __device__ __forceinline__ T make(__nv_bfloat16 a, __nv_bfloat16 b) { return __halves2bfloat162(a, b); } };
template <> struct Pair16<__half> { typedef __half2 T; static __device__ __forceinline__ T make(__half a, __half b) { return __halves2half2(a, b); } };

/* The FP32 correction pass: the vertex update (pageRank.c:1055-1069, fused
 * with the contribution pass :1026-1033) for 16-bit storage.  dsum[v] is
 * the gathered (pull) or scattered (push) sum of the in-neighbours' stored
 * deltas; S[v] is the FP32 sum of everything gathered so far (the sum of
 * the in-neighbours' stored contributions), chat[v] the FP32 value of
 * everything v has stored so far.  rank' = 0.15 + 0.85 * S, the next stored
 * delta is round16(contrib' - chat): what one iteration's rounding lost is
 * sent in the next, so the ranks carry only the rounding of the last delta,
 * which shrinks as the iteration converges.
 * A thread takes two adjacent vertices per step (8-byte loads and stores of
 * every FP32 array, one 4-byte store of the two deltas): the pass moves 34 B
 * per vertex over six arrays, and one vertex per step left too few loads in
 * flight to cover DRAM latency.  Every array is a whole allocation (8-byte
 * aligned); an odd last vertex is taken on its own. */
template <int K>
__global__ void k_pr_update_delta(PrCommon c, float init, float *__restrict__ dsum, float *__restrict__ S,
                                  float *__restrict__ chat, typename Fmt<K>::CT *__restrict__ qout)
{
    typedef typename Fmt<K>::CT CT;
    pdl_wait();
    if (c.skip()) return;
    DeltaStep<K> st{c.base, c.damp, init, c.rec[c.it].qinv, c.eps_f,
                    K == K_F16 ? f16_scale_exp(c.rec[c.it].maxbits) : 0, c.it == 0, 0.0, 0u, 0u};
    float *__restrict__ rank = c.rank;
    const uint32_t *__restrict__ outdeg = c.outdeg;
    const uint32_t P = c.V >> 1, stride = gridDim.x * blockDim.x;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += stride)
    {
        const float2 ds = reinterpret_cast<const float2 *>(dsum)[p];
        float2 s = reinterpret_cast<const float2 *>(S)[p];
        float2 ch = reinterpret_cast<const float2 *>(chat)[p];
        const uint2 deg = reinterpret_cast<const uint2 *>(outdeg)[p];
        if (ds.x != 0.0f || ds.y != 0.0f) reinterpret_cast<float2 *>(dsum)[p] = make_float2(0.0f, 0.0f);
        float2 nr;
        CT q0, q1;
        st(ds.x, s.x, ch.x, deg.x, nr.x, q0);
        st(ds.y, s.y, ch.y, deg.y, nr.y, q1);
        reinterpret_cast<float2 *>(S)[p] = s;
        reinterpret_cast<float2 *>(rank)[p] = nr;
        reinterpret_cast<float2 *>(chat)[p] = ch;
        reinterpret_cast<typename Pair16<CT>::T *>(qout)[p] = Pair16<CT>::make(q0, q1);
    }
    if ((c.V & 1u) && blockIdx.x == 0 && threadIdx.x == 0)
    {
        const uint32_t v = c.V - 1;
        const float ds = dsum[v];
        clear_after_read(&dsum[v], ds);
        float s = S[v], ch = chat[v], nr;
        st(ds, s, ch, outdeg[v], nr, qout[v]);
        S[v] = s;
        rank[v] = nr;
        chat[v] = ch;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) c.rec[c.it + 1].qinv = pow2f(-st.k);
    block_max_bits<256>(st.tmax, &c.rec[c.it + 1].maxbits);
    block_sum2<256>(st.err, st.act);
    if (threadIdx.x == 0) c.reduce(st.err, st.act);
    pdl_trigger();
}

/* ---- data-driven variants (pageRank.c:2810-3300) -------------------------------- */

__global__ void k_dd_contrib(const float *__restrict__ rank, const uint32_t *__restrict__ outdeg, float *cf, uint32_t V,
                             IterRec *rec, uint32_t it)
{
    if (it > 0 && rec[it - 1].active == 0u) return;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
        cf[v] = contrib_of(rank[v], outdeg[v]);
}

/* data-driven pull (pageRank.c:2810-2905): every row is gathered; only
 * worklist vertices update, and a vertex that moved by at least epsilon
 * keeps its new rank and activates its out-neighbours */
struct DdGather
{
    typedef float Acc;
    typedef float Raw;
    const float *cf;
    __device__ __forceinline__ float load(uint32_t, uint32_t u) const { return ldg_val(cf + u); }
    __device__ __forceinline__ float value(float r) const { return r; }
};

__global__ void __launch_bounds__(GG_TILE_NT) k_dd_pull(const uint32_t *__restrict__ off, const uint32_t *__restrict__ adj,
                                                        const uint2 *__restrict__ coord, uint32_t ntiles, uint32_t V,
                                                        float *sums, DdGather op, const IterRec *rec, uint32_t it)
{
    if (it > 0 && rec[it - 1].active == 0u) return;
    warp_pull_sums<GG_TILE_IPT, GG_TILE_WARPS>(off, adj, V, coord, ntiles, sums, op);
}

__global__ void k_dd_update(PrCommon c, float *sums, const uint8_t *__restrict__ wl_curr, uint8_t *wl_next,
                            const uint32_t *__restrict__ out_off, const uint32_t *__restrict__ out_adj)
{
    if (c.skip()) return;
    double err = 0.0;
    uint32_t act = 0;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < c.V; v += gridDim.x * blockDim.x)
    {
        const float sum = sums[v];
        clear_after_read(&sums[v], sum);
        if (!wl_curr[v]) continue;
        float nr = __fadd_rn(c.base, __fmul_rn(c.damp, sum));
        float e = fabsf(__fsub_rn(nr, c.rank[v]));
        err += (double)e;
        if (e >= c.eps_f)
        {
            c.rank[v] = nr;
            for (uint32_t j = out_off[v]; j < out_off[v + 1]; j++) wl_next[out_adj[j]] = 1;
            act++;
        }
    }
    block_sum2<256>(err, act);
    if (threadIdx.x == 0) c.reduce(err, act);
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
    bool use_hot = false; /* pull gather through the hot-vertex table */
    gg_pull_shape shape;  /* launch shape of the FP pull gather */
    uint32_t launches = 0;
    uint32_t gather_launches = 0;
    float gather_ms = 0.0f;
    std::vector<cudaEvent_t> evs;
};

int grid_v(uint32_t V) { int b = (int)((V + 255) / 256); int cap = gg_sm_count() * 8; return b < 1 ? 1 : (b > cap ? cap : b); }

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
    void *c0, *c1, *cf = nullptr, *sums;
    GG_CHECK(gg_work(g, 2, ((size_t)V + 16) * sizeof(CT), &c0));
    GG_CHECK(gg_work(g, 3, ((size_t)V + 16) * sizeof(CT), &c1));
    if (Fmt<K>::quant) GG_CHECK(gg_work(g, 4, ((size_t)V + 16) * sizeof(float), &cf));
    /* row sums, zero between launches (k_pr_update clears what it reads) */
    GG_CHECK(gg_work(g, 5, ((size_t)V + 16) * sizeof(Acc), &sums));
    GG_CUDA(cudaMemsetAsync(sums, 0, ((size_t)V + 16) * sizeof(Acc), R.s));
    CT *cb[2] = {(CT *)c0, (CT *)c1};
    /* 16-bit storage: FP32 running sums and stored-so-far values */
    constexpr bool delta = K == K_BF16 || K == K_F16;
    void *Sb = nullptr, *chb = nullptr;
    if (delta)
    {
        GG_CHECK(gg_work(g, 28, ((size_t)V + 16) * 4, &Sb));
        GG_CHECK(gg_work(g, 29, ((size_t)V + 16) * 4, &chb));
    }

    if constexpr (delta)
        k_pr_init_delta<K><<<grid_v(V), 256, 0, R.s>>>(rank, g->out_deg, V, init, cb[0], (float *)Sb, (float *)chb, rec);
    else
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
        const CT *cin = Fmt<K>::quant ? cb[0] : cb[it & 1];
        GG_CHECK(timed_begin(R));
        int hg = 0;
        const uint32_t hw = R.shape.hot_warps;
        if constexpr (sizeof(Acc) == 4)
            if (R.use_hot && g->hot_cap == hot_entries<K>()) hg = hot_grid<K>(g->hot_tiles.ntiles, hw);
        /* gather and update as programmatic dependent launches (each kernel
         * waits for the one before it; its launch overlaps that kernel's
         * tail), except when they are timed one by one */
        const bool pdl = !R.p->profile;
        if (hg)
        {
            if (pdl)
                GG_CUDA(gg_launch_pdl(k_pr_pull_hot<K>, dim3(hg), dim3(hw * 32), hot_smem_bytes<K>(hw), R.s, g->in_off,
                                      g->hot_adj, g->hot_tiles.coord, g->hot_tiles.ntiles, V, (Acc *)sums, cin,
                                      g->hot_list, g->hot_n, (const IterRec *)rec, it));
            else
                k_pr_pull_hot<K><<<hg, hw * 32, hot_smem_bytes<K>(hw), R.s>>>(
                    g->in_off, g->hot_adj, g->hot_tiles.coord, g->hot_tiles.ntiles, V, (Acc *)sums, cin, g->hot_list,
                    g->hot_n, rec, it);
        }
        else
        {
            const int pg = gg_persistent_grid((const void *)k_pr_pull<K>, t->ntiles, (int)R.shape.ctas);
            if (pdl)
                GG_CUDA(gg_launch_pdl(k_pr_pull<K>, dim3(pg), dim3(GG_TILE_NT), 0, R.s, g->in_off, g->in_adj, t->coord,
                                      t->ntiles, V, (Acc *)sums, PrGather<K>{cin}, (const IterRec *)rec, it));
            else
                k_pr_pull<K><<<pg, GG_TILE_NT, 0, R.s>>>(g->in_off, g->in_adj, t->coord, t->ntiles, V, (Acc *)sums,
                                                        PrGather<K>{cin}, rec, it);
        }
        GG_CHECK(timed_end(R));
        PrCommon c;
        c.rank = rank; c.outdeg = g->out_deg; c.V = V; c.base = base; c.damp = R.p->damp;
        c.eps_f = R.eps_f; c.eps_fl = R.eps_fl; c.rec = rec; c.it = it;
        if constexpr (delta)
        {
            if (pdl)
                GG_CUDA(gg_launch_pdl(k_pr_update_delta<K>, dim3(grid_v(V)), dim3(256), 0, R.s, c, init, (float *)sums,
                                      (float *)Sb, (float *)chb, cb[(it + 1) & 1]));
            else
                k_pr_update_delta<K><<<grid_v(V), 256, 0, R.s>>>(c, init, (float *)sums, (float *)Sb, (float *)chb,
                                                                 cb[(it + 1) & 1]);
        }
        else
        {
            if (pdl)
                GG_CUDA(gg_launch_pdl(k_pr_update<K>, dim3(grid_v(V)), dim3(256), 0, R.s, c, (Acc *)sums,
                                      cb[(it + 1) & 1], (float *)cf));
            else
                k_pr_update<K><<<grid_v(V), 256, 0, R.s>>>(c, (Acc *)sums, cb[(it + 1) & 1], (float *)cf);
        }
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
    /* 16-bit storage: the scatter moves stored deltas (k_pr_update_delta) */
    constexpr bool delta = K == K_BF16 || K == K_F16;
    void *Sb = nullptr, *chb = nullptr;
    if (delta)
    {
        GG_CHECK(gg_work(g, 28, ((size_t)V + 16) * 4, &Sb));
        GG_CHECK(gg_work(g, 29, ((size_t)V + 16) * 4, &chb));
    }
    if constexpr (K == K_Q8Z)
        k_pr_init<K_Q8><<<grid_v(V), 256, 0, R.s>>>(rank, g->out_deg, V, init, nullptr, (float *)cf, rec);
    else if constexpr (delta)
        k_pr_init_delta<K><<<grid_v(V), 256, 0, R.s>>>(rank, g->out_deg, V, init, (CT *)c0, (float *)Sb, (float *)chb,
                                                         rec);
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
            k_pr_update<K_FX64><<<grid_v(V), 256, 0, R.s>>>(c, (unsigned long long *)nx, (unsigned long long *)c0, nullptr);
        else if constexpr (K == K_Q8Z)
            k_pr_update<K_Q8Z><<<grid_v(V), 256, 0, R.s>>>(c, (float *)nx, nullptr, (float *)cf);
        else if constexpr (delta)
            k_pr_update_delta<K><<<grid_v(V), 256, 0, R.s>>>(c, init, (float *)nx, (float *)Sb, (float *)chb, (CT *)c0);
        else
            k_pr_update<K><<<grid_v(V), 256, 0, R.s>>>(c, (float *)nx, (CT *)c0, nullptr);
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
        void *sums;
        GG_CHECK(gg_work(g, 5, ((size_t)V + 16) * 4, &sums));
        GG_CUDA(cudaMemsetAsync(sums, 0, ((size_t)V + 16) * 4, R.s));
        GG_CUDA(cudaMemsetAsync(wa, 1, V, R.s));
        gg_tiles *t;
        GG_CHECK(gg_tiles_get(g, 1, R.s, &t));
        for (uint32_t it = 0; it < iters; it++)
        {
            k_dd_contrib<<<grid_v(V), 256, 0, R.s>>>(rank, g->out_deg, (float *)cf, V, rec, it);
            PrCommon c;
            c.rank = rank; c.outdeg = g->out_deg; c.V = V; c.base = base; c.damp = R.p->damp;
            c.eps_f = R.eps_f; c.eps_fl = R.eps_fl; c.rec = rec; c.it = it;
            GG_CHECK(timed_begin(R));
            k_dd_pull<<<gg_persistent_grid((const void *)k_dd_pull, t->ntiles, GG_PULL_CTAS_PER_SM), GG_TILE_NT, 0, R.s>>>(
                g->in_off, g->in_adj, t->coord, t->ntiles, V, (float *)sums, DdGather{(const float *)cf}, rec, it);
            GG_CHECK(timed_end(R));
            k_dd_update<<<grid_v(V), 256, 0, R.s>>>(c, (float *)sums, wl[it & 1], wl[(it + 1) & 1], g->out_off, g->out_adj);
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

/* every launch of one PageRank run, queued on R.s */
gg_status pagerank_enqueue(Run &R, const gg_pr_params *p, IterRec *rec, float *rank, void *sum_v, uint32_t ngraphs,
                           const uint32_t *voff)
{
    const uint32_t V = R.g->V, iters = p->max_iterations;
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
        if (ngraphs)
            k_pr_finalize_seg<<<grid_v(V), 256, 0, R.s>>>(rank, V, voff, ngraphs, (double *)sum_v);
        else
            GG_CUDA(gg_launch_pdl(k_pr_finalize, dim3(grid_v(V)), dim3(256), 0, R.s, rank, V,
                                  p->init_one_over_n ? 0 : 1, (double *)sum_v));
        R.launches++;
        GG_CUDA(cudaGetLastError());
    }
    return GG_OK;
}


/* many graphs, one CTA per graph, every iteration in one launch (graphs.cu):
 * FP32 pull; per-graph stop; the result reports the largest iteration count
 * and the sum of the active counts of graphs that ran out of iterations */
gg_status graphs_impl(gg_graph *g, const gg_pr_params *p, float *ranks, gg_pr_result *r, void *stream,
                      uint32_t ngraphs, const uint32_t *h_voff)
{
    cudaStream_t s = gg_stream(g, stream);
    const uint32_t V = g->V;
    const gg_graphs_config cfg = gg_graphs_choice(g, ngraphs);
    GG_CHECK(gg_graphs_prepare(g, ngraphs, h_voff, (uint32_t)gg_graphs_tile_items(cfg), s));
    void *rank_v, *stat, *sum_v;
    GG_CHECK(gg_work(g, 0, ((size_t)V + 16) * 4, &rank_v));
    GG_CHECK(gg_work(g, 23, 64 + (size_t)ngraphs * 16, &stat));
    GG_CHECK(gg_work(g, 10, 64, &sum_v));
    uint32_t *counter = (uint32_t *)stat;
    uint32_t *iters = (uint32_t *)((char *)stat + 64);
    uint32_t *active = iters + ngraphs;
    double *err = (double *)(active + ngraphs + (ngraphs & 1));
    GG_CUDA(cudaMemsetAsync(sum_v, 0, 64, s));
    /* vertices outside every graph keep rank 0 */
    if (h_voff[0] > 0 || h_voff[ngraphs] < V) GG_CUDA(cudaMemsetAsync(rank_v, 0, (size_t)V * 4, s));
    gg_pr_result res;
    memset(&res, 0, sizeof(res));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (p->profile)
    {
        GG_CHECK(gg_event_at(g, 0, &e0));
        GG_CHECK(gg_event_at(g, 1, &e1));
        GG_CUDA(cudaEventRecord(e0, s));
    }
    GG_CHECK(gg_graphs_launch(g, cfg, ngraphs, p, gg_float_ceil(p->epsilon), (float *)rank_v, counter, iters, active,
                              err, s));
    if (p->profile) GG_CUDA(cudaEventRecord(e1, s));
    k_pr_finalize<<<grid_v(V), 256, 0, s>>>((float *)rank_v, V, 0, (double *)sum_v);
    GG_CUDA(cudaGetLastError());
    std::vector<uint32_t> h_it(2 * (size_t)ngraphs);
    std::vector<double> h_err(ngraphs);
    double sum = 0.0;
    /* a bounded wait first: a copy to pageable memory would block until the
     * launch ends, however long that is */
    GG_CHECK(gg_wait(s));
    GG_CUDA(cudaMemcpyAsync(h_it.data(), iters, (size_t)ngraphs * 8, cudaMemcpyDeviceToHost, s));
    GG_CUDA(cudaMemcpyAsync(h_err.data(), err, (size_t)ngraphs * 8, cudaMemcpyDeviceToHost, s));
    GG_CUDA(cudaMemcpyAsync(&sum, sum_v, 8, cudaMemcpyDeviceToHost, s));
    if (ranks && V) GG_CHECK(gg_copy_d2h(ranks, rank_v, (size_t)V * 4, s));
    GG_CHECK(gg_wait(s));
    for (uint32_t i = 0; i < ngraphs; i++)
    {
        res.iterations = std::max(res.iterations, h_it[i]);
        if (h_it[i] >= p->max_iterations) res.active += h_it[ngraphs + i];
        res.error_total = std::max(res.error_total, h_err[i]);
    }
    res.rank_sum = sum;
    res.launches = 2;
    res.gather_launches = 1;
    if (p->profile) res.gather_ms = gg_event_ms(e0, e1);
    g->last_ranks = (const float *)rank_v;
    g->graphs_iters = iters;
    g->graphs_n = ngraphs;
    if (r) *r = res;
    return GG_OK;
}

/* one PageRank run; with ngraphs > 0 the mapping is the union of ngraphs
 * graphs (vertex ranges h_voff[g] .. h_voff[g+1]) and the final
 * normalisation divides each vertex by its own graph's vertex count */
gg_status pagerank_impl(gg_graph *g, const gg_pr_params *p, float *ranks, gg_pr_result *r, void *stream,
                        uint32_t ngraphs, const uint32_t *h_voff)
{
    GgRange range(ngraphs ? "gg_pagerank_batch" : "gg_pagerank");
    if (!g || !p) return gg_fail(GG_ERR_INVALID, "NULL argument");
    if (p->mode > 13) return gg_fail(GG_ERR_INVALID, "unknown PageRank mode");
    if (p->storage > 2) return gg_fail(GG_ERR_INVALID, "unknown storage");
    if (ngraphs && p->mode == GG_PR_PULL && p->storage == GG_STORE_F32 && !(p->flags & GG_PR_BATCH_UNION))
    {
        if (!g->in_off || !g->out_deg) return gg_fail(GG_ERR_INVALID, "pull PageRank needs GG_MAP_IN");
        /* an epsilon stop needs the many-graphs kernel (every graph stops on
         * its own; the union stops when all have converged); without one
         * every graph runs all iterations either way and the strategy
         * decides: the union pull by default (faster on every R-MAT mix
         * measured), the many-graphs kernel when set or tuned so */
        const gg_graphs_config cfg = gg_graphs_choice(g, ngraphs);
        if (p->epsilon > 0.0 || cfg.strategy == 1) return graphs_impl(g, p, ranks, r, stream, ngraphs, h_voff);
    }
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

    void *rank_v, *rec_v, *sum_v, *voff_v = nullptr;
    GG_CHECK(gg_work(g, 0, ((size_t)V + 16) * 4, &rank_v));
    GG_CHECK(gg_work(g, 1, ((size_t)iters + 2) * sizeof(IterRec), &rec_v));
    GG_CHECK(gg_work(g, 10, 64, &sum_v));
    IterRec *rec = (IterRec *)rec_v;
    float *rank = (float *)rank_v;
    if (ngraphs)
    {
        GG_CHECK(gg_work(g, 23, ((size_t)ngraphs + 1) * 4, &voff_v));
        GG_CUDA(cudaMemcpyAsync(voff_v, h_voff, ((size_t)ngraphs + 1) * 4, cudaMemcpyHostToDevice, R.s));
    }

    /* the hot-vertex table for the FP pull modes (prepared before any
     * capture: preparation reads back to the host) */
    gg_tune_lookup(g, R.s);
    R.shape = g->pr_shape;
    const bool hot_default = R.shape.hot == 2 ? V >= (1u << 20) : R.shape.hot == 1;
    if (p->mode == GG_PR_PULL && !(p->flags & GG_PR_HOT_OFF) && ((p->flags & GG_PR_HOT_ON) || hot_default) &&
        V < GG_HOT_FLAG && V > 0)
    {
        const uint32_t cap = GG_HOT_TABLE_BYTES / (p->storage == GG_STORE_F32 ? 4u : 2u);
        GG_CHECK(gg_hot_prepare(g, R.s, cap < GG_HOT_ENTRIES ? cap : GG_HOT_ENTRIES));
        R.use_hot = true;
    }

    /* with GG_PR_CUDA_GRAPH everything from here to the final normalisation
     * is captured into one CUDA graph (relaxed capture: buffers first used
     * inside it are allocated during the capture) and instantiated; the
     * instance stays with the mapping and is launched again by calls with
     * the same parameters while no device memory of the mapping has been
     * freed since (the buffers it writes are then the same) */
    const bool as_graph = (p->flags & GG_PR_CUDA_GRAPH) != 0;
    gg_status st = GG_OK;
    if (as_graph)
    {
        struct Key
        {
            uint32_t mode, storage, iters, init, flags, ngraphs, use_hot, V, E, ctas, hot_warps;
            float damp;
            double eps;
        } key;
        static_assert(sizeof(Key) <= sizeof(g->pr_key), "PageRank graph key");
        memset(&key, 0, sizeof(key));
        key.mode = p->mode; key.storage = p->storage; key.iters = iters; key.init = p->init_one_over_n;
        key.flags = p->flags; key.ngraphs = ngraphs; key.use_hot = R.use_hot ? 1u : 0u; key.V = V; key.E = g->E;
        key.ctas = R.shape.ctas; key.hot_warps = R.shape.hot_warps;
        key.damp = p->damp; key.eps = p->epsilon;
        if (g->pr_exec && g->pr_gen == g->mem_gen && memcmp(g->pr_key, &key, sizeof(key)) == 0)
        {
            GG_CUDA(cudaGraphLaunch(g->pr_exec, R.s));
            R.launches = g->pr_launches;
            R.gather_launches = g->pr_gather_launches;
        }
        else
        {
            if (g->pr_exec)
            {
                cudaGraphExecDestroy(g->pr_exec);
                g->pr_exec = nullptr;
            }
            GG_CUDA(cudaStreamBeginCapture(R.s, cudaStreamCaptureModeRelaxed));
            st = pagerank_enqueue(R, p, rec, rank, sum_v, ngraphs, (const uint32_t *)voff_v);
            cudaGraph_t graph = nullptr;
            cudaError_t e = cudaStreamEndCapture(R.s, &graph);
            if (st == GG_OK && e != cudaSuccess) st = gg_cuda_fail(e, "cudaStreamEndCapture");
            cudaGraphExec_t exec = nullptr;
            if (st == GG_OK)
            {
                e = cudaGraphInstantiate(&exec, graph, 0);
                if (e != cudaSuccess) st = gg_cuda_fail(e, "cudaGraphInstantiate");
            }
            if (graph) cudaGraphDestroy(graph);
            if (st == GG_OK)
            {
                e = cudaGraphLaunch(exec, R.s);
                if (e != cudaSuccess) st = gg_cuda_fail(e, "cudaGraphLaunch");
            }
            if (st == GG_OK)
            {
                g->pr_exec = exec;
                memcpy(g->pr_key, &key, sizeof(key));
                g->pr_gen = g->mem_gen;
                g->pr_launches = R.launches;
                g->pr_gather_launches = R.gather_launches;
            }
            else if (exec)
                cudaGraphExecDestroy(exec);
        }
    }
    else
        st = pagerank_enqueue(R, p, rec, rank, sum_v, ngraphs, (const uint32_t *)voff_v);
    if (st != GG_OK) return st;

    std::vector<IterRec> h(iters + 2);
    double sum = 0.0;
    /* a bounded wait first: a copy to pageable memory would block until the
     * iterations end, however long that is; the rank destination's pages are
     * made resident while the iterations run */
    if (ranks && V) gg_host_dst_prepare(ranks, (size_t)V * 4);
    GG_CHECK(gg_wait(R.s));
    GG_CUDA(cudaMemcpyAsync(h.data(), rec, ((size_t)iters + 2) * sizeof(IterRec), cudaMemcpyDeviceToHost, R.s));
    GG_CUDA(cudaMemcpyAsync(&sum, sum_v, sizeof(double), cudaMemcpyDeviceToHost, R.s));
    if (ranks && V) GG_CHECK(gg_copy_d2h(ranks, rank, (size_t)V * 4, R.s));
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
    res.hot_table = R.use_hot ? 1u : 0u;
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

} // namespace

extern "C" gg_status gg_pagerank(gg_graph *g, const gg_pr_params *p, float *ranks, gg_pr_result *r, void *stream)
{
    return pagerank_impl(g, p, ranks, r, stream, 0, nullptr);
}

extern "C" gg_status gg_pagerank_batch(gg_graph *g, const gg_pr_params *p, uint32_t ngraphs, const uint32_t *vertex_off,
                                       float *ranks, gg_pr_result *r, void *stream)
{
    if (!g || !p || !vertex_off || ngraphs == 0) return gg_fail(GG_ERR_INVALID, "NULL argument or no graphs");
    if (p->init_one_over_n)
        return gg_fail(GG_ERR_INVALID, "batched PageRank uses the reference formulation (init_one_over_n = 0)");
    if (vertex_off[0] != 0 || vertex_off[ngraphs] != g->V)
        return gg_fail(GG_ERR_INVALID, "vertex_off must run from 0 to the mapping's vertex count");
    for (uint32_t i = 0; i < ngraphs; i++)
        if (vertex_off[i + 1] <= vertex_off[i]) return gg_fail(GG_ERR_INVALID, "every graph needs a vertex");
    return pagerank_impl(g, p, ranks, r, stream, ngraphs, vertex_off);
}

extern "C" const float *gg_pagerank_device_ranks(const gg_graph *g) { return g ? g->last_ranks : nullptr; }
