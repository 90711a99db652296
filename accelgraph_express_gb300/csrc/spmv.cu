/*
 * SpMV on CSR (02_capi_graph/src/algorithms/capi/SPMV.c:594-1135) on one GPU.
 *
 *   pull  (mode 0): y[v] = sum over in-edges (u,v) of w(u,v)*x[u]; the
 *                   merge-path tile gather over the CSC, recomputed every
 *                   iteration like the FPGA CU run per iteration (:712-718)
 *   push  (mode 1): y[dst] += w*x[src] over out-edges with FP32 atomics,
 *                   accumulating across iterations (:795-820)
 *   pull fixed (2): Q16.16 operands, (x*w) >> 16 summed in 64 bits
 *                   (cu_SPMV/CSR/PULL/FixedPoint/cu/cu_sum_kernel_control.sv:155-184)
 *   push fixed (3): Q32.32, y64 += (w*x) >> 32 (:1080-1093)
 * x and the weights may be stored as BF16/FP16 (FP32 products and sums).
 */
#include <cuda_runtime.h>
#include <cmath>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cstring>
#include <string>
#include <vector>

#include "gg_device.cuh"

namespace {

using namespace gg;

/* the edge term of the pull product: w[e] * x[u] (SPMV.c:735-760) */
template <class T>
struct SpmvGather
{
    typedef float Acc;
    struct Raw { T w, x; };
    const T *w;
    const T *x;
    __device__ __forceinline__ Raw load(uint32_t e, uint32_t u) const { return Raw{ldg_val(w + e), ldg_val(x + u)}; }
    __device__ __forceinline__ float value(const Raw &r) const { return __fmul_rn(to_f32(r.w), to_f32(r.x)); }
};

template <class T>
__global__ void __launch_bounds__(GG_TILE_NT) k_spmv_pull(const uint32_t *__restrict__ off, const uint32_t *__restrict__ adj,
                                                          const uint2 *__restrict__ coord, uint32_t ntiles, uint32_t V,
                                                          float *y, SpmvGather<T> op)
{
    warp_pull_sums<GG_TILE_IPT, GG_TILE_WARPS>(off, adj, V, coord, ntiles, y, op);
}

/* the pull product with the hot-vertex table: x of the flagged in-neighbours
 * comes from shared memory (the same table as the PageRank gather's) */
template <class T>
struct SpmvGatherHot
{
    typedef float Acc;
    typedef typename SpmvGather<T>::Raw Raw;
    const T *w;
    const T *x;
    const T *s_hot;
    __device__ __forceinline__ Raw load(uint32_t e, uint32_t u) const
    {
        const T wv = ldg_val(w + e);
        if (u & GG_HOT_FLAG) return Raw{wv, s_hot[u & ~GG_HOT_FLAG]};
        return Raw{wv, ldg_val(x + u)};
    }
    __device__ __forceinline__ float value(const Raw &r) const { return __fmul_rn(to_f32(r.w), to_f32(r.x)); }
};

template <class T>
__host__ __device__ constexpr size_t spmv_hot_stage_bytes(uint32_t warps)
{
    return (size_t)warps * PullStage<GG_HOT_IPT, float>::BYTES;
}
template <class T>
__host__ __device__ constexpr uint32_t spmv_hot_entries()
{
    return GG_HOT_TABLE_BYTES / sizeof(T) < GG_HOT_ENTRIES ? (uint32_t)(GG_HOT_TABLE_BYTES / sizeof(T)) : GG_HOT_ENTRIES;
}
template <class T>
__host__ __device__ constexpr size_t spmv_hot_smem_bytes(uint32_t warps)
{
    return spmv_hot_stage_bytes<T>(warps) + ((size_t)spmv_hot_entries<T>() * sizeof(T) + 15) / 16 * 16;
}

template <class T>
__global__ void __launch_bounds__(GG_HOT_WARPS * 32, 1)
    k_spmv_pull_hot(const uint32_t *__restrict__ off, const uint32_t *__restrict__ hot_adj,
                    const uint2 *__restrict__ coord, uint32_t ntiles, uint32_t V, float *y, const T *w,
                    const T *__restrict__ x, const uint32_t *__restrict__ hot_list, uint32_t hot_n)
{
    extern __shared__ __align__(16) unsigned char gg_dyn[];
    T *s_hot = reinterpret_cast<T *>(gg_dyn + spmv_hot_stage_bytes<T>(blockDim.x >> 5));
    for (uint32_t i = threadIdx.x; i < hot_n; i += blockDim.x) s_hot[i] = x[hot_list[i]];
    __syncthreads();
    warp_pull_sums_dyn<GG_HOT_IPT>(gg_dyn, off, hot_adj, V, coord, ntiles, y, SpmvGatherHot<T>{w, x, s_hot});
}

/* one CTA of `warps` warps per SM, carve-out sized to its shared memory */
template <class T>
int spmv_hot_grid(uint32_t ntiles, uint32_t warps)
{
    static int ok = -1;
    static uint32_t applied = 0;
    if (ok < 0)
    {
        const size_t most = spmv_hot_smem_bytes<T>(GG_HOT_WARPS);
        cudaError_t e = cudaFuncSetAttribute(k_spmv_pull_hot<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)most);
        ok = e == cudaSuccess ? 1 : 0;
        if (!ok) cudaGetLastError();
    }
    if (!ok) return 0;
    if (applied != warps)
    {
        int dev = 0, smem_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
        if (smem_sm > 0)
        {
            const int pct = (int)ceil(100.0 * (double)(spmv_hot_smem_bytes<T>(warps) + 1024) / (double)smem_sm);
            if (cudaFuncSetAttribute(k_spmv_pull_hot<T>, cudaFuncAttributePreferredSharedMemoryCarveout,
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

/* fixed-point pull (SPMV.c:775-815): x in Q16.16, weights converted per
 * edge, products truncated to Q16.16 and summed exactly in 64 bits */
struct SpmvFxGather
{
    typedef unsigned long long Acc;
    struct Raw { float w; uint32_t x; };
    const float *w;
    const uint32_t *x32;
    __device__ __forceinline__ Raw load(uint32_t e, uint32_t u) const { return Raw{ldg_val(w + e), ldg_val(x32 + u)}; }
    __device__ __forceinline__ unsigned long long value(const Raw &r) const
    {
        return ((unsigned long long)r.x * fx_from_float(r.w, 65536.0, 0xffffffffu)) >> 16;
    }
};

__global__ void __launch_bounds__(GG_TILE_NT) k_spmv_pull_fx(const uint32_t *__restrict__ off, const uint32_t *__restrict__ adj,
                                                             const uint2 *__restrict__ coord, uint32_t ntiles, uint32_t V,
                                                             unsigned long long *y64, SpmvFxGather op)
{
    warp_pull_sums<GG_TILE_IPT, GG_TILE_WARPS>(off, adj, V, coord, ntiles, y64, op);
}

/* y = Q16.16 sums as float; clears the sums for the next product */
__global__ void k_spmv_fx_pull_out(unsigned long long *y64, float *y, uint32_t V)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
    {
        const unsigned long long s = y64[v];
        y[v] = fx_to_float(s, 1.0 / 65536.0);
        clear_after_read(&y64[v], s);
    }
}

template <class T>
__global__ void __launch_bounds__(GG_TILE_NT) k_spmv_push(const uint32_t *__restrict__ off, const uint32_t *__restrict__ adj,
                                                          const uint2 *__restrict__ coord, uint32_t ntiles, uint32_t V,
                                                          const T *w, const T *x, float *y)
{
    struct Op
    {
        typedef float RowVal;
        const T *w;
        const T *x;
        float *y;
        __device__ __forceinline__ float row_value(uint32_t r) const { return to_f32(x[r]); }
        __device__ __forceinline__ void scatter(float xv, uint32_t e, uint32_t dst) const
        {
            atomicAdd(&y[dst], __fmul_rn(to_f32(w[e]), xv));
        }
    } op{w, x, y};
    warp_push<GG_TILE_IPT, GG_TILE_WARPS>(off, adj, V, coord, ntiles, op);
}

__global__ void __launch_bounds__(GG_TILE_NT) k_spmv_push_fx(const uint32_t *__restrict__ off, const uint32_t *__restrict__ adj,
                                                             const uint2 *__restrict__ coord, uint32_t ntiles, uint32_t V,
                                                             const float *w, const unsigned long long *x64,
                                                             unsigned long long *y64)
{
    struct Op
    {
        typedef unsigned long long RowVal;
        const float *w;
        const unsigned long long *x64;
        unsigned long long *y64;
        __device__ __forceinline__ unsigned long long row_value(uint32_t r) const { return x64[r]; }
        __device__ __forceinline__ void scatter(unsigned long long xv, uint32_t e, uint32_t dst) const
        {
            atomicAdd(&y64[dst], fx64_mul(fx64_from_double((double)w[e]), xv));
        }
    } op{w, x64, y64};
    warp_push<GG_TILE_IPT, GG_TILE_WARPS>(off, adj, V, coord, ntiles, op);
}

/* x[v] = 1/outdeg(v), or 0.001 when 0 (SPMV.c:696-701), unless given; the
 * stored copy in the chosen storage and the fixed-point copies */
template <class T>
__global__ void k_spmv_x(const uint32_t *__restrict__ outdeg, const float *xin, float *xf, T *xs, uint32_t *x32,
                         unsigned long long *x64, float *y, uint32_t V)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
    {
        float xv;
        if (xin)
            xv = xin[v];
        else
        {
            uint32_t d = outdeg[v];
            xv = d ? __fdiv_rn(1.0f, __uint2float_rn(d)) : 0.001f;
        }
        xf[v] = xv;
        if (xs) xs[v] = from_f32<T>(xv);
        if (x32) x32[v] = fx_from_float(xv, 65536.0, 0xffffffffu);
        if (x64) x64[v] = fx64_from_double((double)xv);
        y[v] = 0.0f;
    }
}

__global__ void k_spmv_fx64_out(const unsigned long long *y64, float *y, uint32_t V)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
        y[v] = __double2float_rn(fx64_to_double(y64[v]));
}

/* sum of round2(y) as the reference prints it (SPMV.c:727-730) */
__global__ void k_spmv_checksum(const float *y, uint32_t V, double *out)
{
    double s = 0.0;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
    {
        double t = __dadd_rn((double)__fmul_rn(y[v], 100.0f), 0.5);
        s += (double)(int)t / 100.0;
    }
    uint32_t dummy = 0;
    block_sum2<256>(s, dummy);
    if (threadIdx.x == 0 && s != 0.0) atomicAdd(out, s);
}

int grid_v(uint32_t V) { int b = (int)((V + 255) / 256); int cap = gg_sm_count() * 8; return b < 1 ? 1 : (b > cap ? cap : b); }

template <class T>
gg_status spmv_fp(gg_graph *g, const gg_spmv_params *p, const float *x_dev, float *xf, float *y, cudaStream_t s,
                  uint32_t &launches, uint32_t &timed, std::vector<cudaEvent_t> &evs)
{
    const uint32_t V = g->V;
    const bool pull = p->mode == GG_SPMV_PULL;
    gg_tiles *t;
    GG_CHECK(gg_tiles_get(g, pull ? 1 : 0, s, &t));
    void *xs = nullptr;
    const T *w;
    if constexpr (sizeof(T) == 4)
    {
        w = (const T *)(pull ? g->in_w : g->out_w);
    }
    else
    {
        const void *w16;
        GG_CHECK(gg_weights16(g, pull ? 1 : 0, p->storage, s, &w16));
        w = (const T *)w16;
        GG_CHECK(gg_work(g, 12, ((size_t)V + 16) * sizeof(T), &xs));
    }
    k_spmv_x<T><<<grid_v(V), 256, 0, s>>>(g->out_deg, x_dev, xf, (T *)xs, nullptr, nullptr, y, V);
    launches++;
    const T *xv = sizeof(T) == 4 ? (const T *)xf : (const T *)xs;
    /* the hot-vertex table (as for the PageRank pull): by default from 1M vertices */
    bool use_hot = false;
    gg_tune_lookup(g, s);
    const gg_pull_shape shape = g->spmv_shape;
    const bool hot_default = shape.hot == 2 ? V >= (1u << 20) : shape.hot == 1;
    if (pull && !(p->flags & GG_PR_HOT_OFF) && ((p->flags & GG_PR_HOT_ON) || hot_default) && V < GG_HOT_FLAG)
    {
        GG_CHECK(gg_hot_prepare(g, s, spmv_hot_entries<T>()));
        use_hot = g->hot_cap == spmv_hot_entries<T>();
    }
    for (uint32_t it = 0; it < p->iterations; it++)
    {
        if (p->profile)
        {
            cudaEvent_t e;
            GG_CHECK(gg_event_at(g, (uint32_t)evs.size(), &e));
            GG_CUDA(cudaEventRecord(e, s));
            evs.push_back(e);
        }
        if (pull)
        {
            /* y is the row-sum array: zero, then the gather stores rows and
             * adds the partials of rows spanning tiles */
            GG_CUDA(cudaMemsetAsync(y, 0, (size_t)V * sizeof(float), s));
            const int hg = use_hot ? spmv_hot_grid<T>(g->hot_tiles.ntiles, shape.hot_warps) : 0;
            if (hg)
                k_spmv_pull_hot<T><<<hg, shape.hot_warps * 32, spmv_hot_smem_bytes<T>(shape.hot_warps), s>>>(
                    g->in_off, g->hot_adj, g->hot_tiles.coord, g->hot_tiles.ntiles, V, y, w, xv, g->hot_list, g->hot_n);
            else
                k_spmv_pull<T><<<gg_persistent_grid((const void *)k_spmv_pull<T>, t->ntiles, (int)shape.ctas),
                                 GG_TILE_NT, 0, s>>>(g->in_off, g->in_adj, t->coord, t->ntiles, V, y, SpmvGather<T>{w, xv});
        }
        else
            k_spmv_push<T><<<gg_persistent_grid((const void *)k_spmv_push<T>, t->ntiles), GG_TILE_NT, 0, s>>>(
                g->out_off, g->out_adj, t->coord, t->ntiles, V, w, xv, y);
        if (p->profile)
        {
            cudaEvent_t e;
            GG_CHECK(gg_event_at(g, (uint32_t)evs.size(), &e));
            GG_CUDA(cudaEventRecord(e, s));
            evs.push_back(e);
        }
        launches++;
        timed++;
    }
    GG_CUDA(cudaGetLastError());
    return GG_OK;
}

} // namespace

extern "C" gg_status gg_spmv(gg_graph *g, const gg_spmv_params *p, const float *x, float *x_out, float *y,
                             gg_spmv_result *r, void *stream)
{
    GgRange range("gg_spmv");
    if (!g || !p) return gg_fail(GG_ERR_INVALID, "NULL argument");
    if (p->mode > 3) return gg_fail(GG_ERR_INVALID, "unknown SpMV mode");
    if (p->storage > 2) return gg_fail(GG_ERR_INVALID, "unknown storage");
    const bool pull = p->mode == GG_SPMV_PULL || p->mode == GG_SPMV_PULL_FX;
    if (pull && (!g->in_off || !g->in_w)) return gg_fail(GG_ERR_INVALID, "pull SpMV needs GG_MAP_IN|GG_MAP_IN_W");
    if (!pull && (!g->out_off || !g->out_w)) return gg_fail(GG_ERR_INVALID, "push SpMV needs GG_MAP_OUT|GG_MAP_OUT_W");
    if (!g->out_deg) return gg_fail(GG_ERR_INVALID, "mapping has no out-degrees");
    cudaStream_t s = gg_stream(g, stream);
    const uint32_t V = g->V;
    gg_spmv_result res;
    memset(&res, 0, sizeof(res));
    void *xf, *yv, *xin = nullptr, *chk;
    GG_CHECK(gg_work(g, 0, ((size_t)V + 16) * 4, &xf));
    GG_CHECK(gg_work(g, 11, ((size_t)V + 16) * 4, &yv));
    GG_CHECK(gg_work(g, 10, 64, &chk));
    GG_CUDA(cudaMemsetAsync(chk, 0, 64, s));
    if (x)
    {
        GG_CHECK(gg_work(g, 13, ((size_t)V + 16) * 4, &xin));
        GG_CUDA(cudaMemcpyAsync(xin, x, (size_t)V * 4, cudaMemcpyHostToDevice, s));
    }
    std::vector<cudaEvent_t> evs;
    uint32_t launches = 0, timed = 0;
    if (V > 0)
    {
        if (p->mode == GG_SPMV_PULL || p->mode == GG_SPMV_PUSH)
        {
            gg_status st = p->storage == GG_STORE_BF16
                               ? spmv_fp<__nv_bfloat16>(g, p, (const float *)xin, (float *)xf, (float *)yv, s, launches, timed, evs)
                           : p->storage == GG_STORE_F16
                               ? spmv_fp<__half>(g, p, (const float *)xin, (float *)xf, (float *)yv, s, launches, timed, evs)
                               : spmv_fp<float>(g, p, (const float *)xin, (float *)xf, (float *)yv, s, launches, timed, evs);
            if (st != GG_OK) return st;
        }
        else
        {
            gg_tiles *t;
            GG_CHECK(gg_tiles_get(g, pull ? 1 : 0, s, &t));
            void *xq, *y64 = nullptr;
            GG_CHECK(gg_work(g, 12, ((size_t)V + 16) * 8, &xq));
            GG_CHECK(gg_work(g, 14, ((size_t)V + 16) * 8, &y64));
            GG_CUDA(cudaMemsetAsync(y64, 0, ((size_t)V + 16) * 8, s));
            k_spmv_x<float><<<grid_v(V), 256, 0, s>>>(g->out_deg, (const float *)xin, (float *)xf, nullptr,
                                                      pull ? (uint32_t *)xq : nullptr,
                                                      pull ? nullptr : (unsigned long long *)xq, (float *)yv, V);
            launches++;
            for (uint32_t it = 0; it < p->iterations; it++)
            {
                if (p->profile)
                {
                    cudaEvent_t e;
                    GG_CHECK(gg_event_at(g, (uint32_t)evs.size(), &e));
                    GG_CUDA(cudaEventRecord(e, s));
                    evs.push_back(e);
                }
                if (pull)
                {
                    k_spmv_pull_fx<<<gg_persistent_grid((const void *)k_spmv_pull_fx, t->ntiles, GG_PULL_CTAS_PER_SM), GG_TILE_NT, 0, s>>>(
                        g->in_off, g->in_adj, t->coord, t->ntiles, V, (unsigned long long *)y64,
                        SpmvFxGather{g->in_w, (const uint32_t *)xq});
                    k_spmv_fx_pull_out<<<grid_v(V), 256, 0, s>>>((unsigned long long *)y64, (float *)yv, V);
                    launches++;
                }
                else
                    k_spmv_push_fx<<<gg_persistent_grid((const void *)k_spmv_push_fx, t->ntiles), GG_TILE_NT, 0, s>>>(
                        g->out_off, g->out_adj, t->coord, t->ntiles, V, g->out_w, (const unsigned long long *)xq,
                        (unsigned long long *)y64);
                if (p->profile)
                {
                    cudaEvent_t e;
                    GG_CHECK(gg_event_at(g, (uint32_t)evs.size(), &e));
                    GG_CUDA(cudaEventRecord(e, s));
                    evs.push_back(e);
                }
                launches++;
                timed++;
            }
            if (!pull)
            {
                k_spmv_fx64_out<<<grid_v(V), 256, 0, s>>>((const unsigned long long *)y64, (float *)yv, V);
                launches++;
            }
        }
        k_spmv_checksum<<<grid_v(V), 256, 0, s>>>((const float *)yv, V, (double *)chk);
        launches++;
        GG_CUDA(cudaGetLastError());
    }
    double checksum = 0.0;
    GG_CHECK(gg_wait(s)); /* bounded, before a copy to pageable memory */
    GG_CUDA(cudaMemcpyAsync(&checksum, chk, 8, cudaMemcpyDeviceToHost, s));
    if (y && V) GG_CHECK(gg_copy_d2h(y, yv, (size_t)V * 4, s));
    if (x_out && V) GG_CHECK(gg_copy_d2h(x_out, xf, (size_t)V * 4, s));
    GG_CHECK(gg_wait(s));
    res.checksum = checksum;
    res.launches = launches;
    res.spmv_launches = timed;
    if (p->profile)
        for (size_t i = 0; i + 1 < evs.size(); i += 2) res.spmv_ms += gg_event_ms(evs[i], evs[i + 1]);
    if (r) *r = res;
    return GG_OK;
}

/* ---- allocation-free SpMV pull -------------------------------------------------
 *
 * For callers that must not allocate GPU memory: code running inside an
 * allocator-free section (a host memory manager or plugin host that owns
 * every device allocation and forbids cudaMalloc/cudaFree from plugins, a
 * real-time loop where an allocation could block or fragment, or a process
 * whose device memory is fully reserved up front).  gg_spmv needs a
 * gg_graph mapping and work buffers that the runtime allocates; this entry
 * point instead takes the caller's device arrays and keeps its scratch (the
 * merge-path tile coordinates) in the file-scope array below, which exists
 * on every GPU that loads the library until the process exits; partial sums
 * of rows spanning tiles accumulate in the caller's y.
 */
#define GG_NOALLOC_SCRATCH_BYTES (4u << 20)

static __device__ __align__(256) unsigned char g_noalloc_scratch[GG_NOALLOC_SCRATCH_BYTES];

namespace {

size_t noalloc_coord_bytes(uint32_t ntiles) { return (((size_t)ntiles + 1) * sizeof(uint2) + 255) / 256 * 256; }

/* [a, a + an) and [b, b + bn) share a byte */
bool noalloc_overlap(const void *a, size_t an, const void *b, size_t bn)
{
    const uintptr_t pa = (uintptr_t)a, pb = (uintptr_t)b;
    return an && bn && pa < pb + bn && pb < pa + an;
}

} // namespace

extern "C" uint64_t gg_spmv_pull_noalloc_max_items(void)
{
    /* the largest V + E whose tile coordinates fit: (ntiles+1) of 8 bytes,
     * rounded to 256 */
    uint64_t lo = 0, hi = (uint64_t)GG_NOALLOC_SCRATCH_BYTES / 8 * GG_TILE_ITEMS;
    while (lo < hi)
    {
        const uint64_t mid = (lo + hi + 1) / 2;
        const uint64_t nt = (mid + GG_TILE_ITEMS - 1) / GG_TILE_ITEMS;
        if (noalloc_coord_bytes((uint32_t)nt) <= GG_NOALLOC_SCRATCH_BYTES)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

extern "C" gg_status gg_spmv_pull_noalloc(uint32_t V, uint32_t E, const uint32_t *in_off, const uint32_t *in_src,
                                          const float *w, const float *x, float *y, void *stream)
{
    if (V == 0) return GG_OK;
    if (!in_off || !x || !y || !w || (E && !in_src)) return gg_fail(GG_ERR_INVALID, "NULL device array");
    const uint64_t items = (uint64_t)V + E;
    const uint64_t max_items = gg_spmv_pull_noalloc_max_items();
    if (items > max_items)
        return gg_fail(GG_ERR_INVALID, "gg_spmv_pull_noalloc: V + E = " + std::to_string(items) +
                                           " exceeds the scratch limit of " + std::to_string(max_items) +
                                           " (4 MiB of tile scratch); use gg_spmv");
    /* y is written while the others are read (x through the read-only
     * path): an overlap would silently corrupt the product */
    const size_t vb = (size_t)V * sizeof(float), eb = (size_t)E * sizeof(float);
    if (noalloc_overlap(y, vb, x, vb) || noalloc_overlap(y, vb, w, eb) || noalloc_overlap(y, vb, in_src, eb) ||
        noalloc_overlap(y, vb, in_off, vb + sizeof(uint32_t)))
        return gg_fail(GG_ERR_INVALID, "gg_spmv_pull_noalloc: y overlaps x, w, in_off or in_src");
    /* The host-side name of the array is not a device address: ask the
     * runtime for it on every call, in the context current now.  A cached
     * address would go stale when the context it came from is reset or when
     * the caller switches to another context of the same device; the lookup
     * is host-side and queues no work.  The first call in a context loads the
     * library's kernels into it. */
    void *base = nullptr;
    GG_CUDA(cudaGetSymbolAddress(&base, g_noalloc_scratch));
    const uint32_t ntiles = (uint32_t)((items + GG_TILE_ITEMS - 1) / GG_TILE_ITEMS);
    uint2 *coord = (uint2 *)base;
    cudaStream_t s = (cudaStream_t)stream;
    /* the coordinates are rewritten on every call; y is the row-sum array
     * and starts at zero (rows spanning tiles are added into it) */
    GG_CHECK(gg_launch_tile_coords(in_off, V, E, ntiles, coord, s));
    GG_CUDA(cudaMemsetAsync(y, 0, (size_t)V * sizeof(float), s));
    k_spmv_pull<float><<<gg_persistent_grid((const void *)k_spmv_pull<float>, ntiles, GG_PULL_CTAS_PER_SM), GG_TILE_NT, 0, s>>>(
        in_off, in_src, coord, ntiles, V, y, SpmvGather<float>{w, x});
    GG_CUDA(cudaGetLastError());
    return GG_OK;
}
