/*
 * The ceilings the PageRank / SpMV pull gather is measured against: random
 * 4-byte gathers per second, from hashed indices (no index traffic), every
 * thread summing 4096 values, when the values come from
 *   - the shared memory of an 8-CTA thread-block cluster (184 KB per CTA),
 *   - the CTA's own shared memory,
 *   - global memory, a 1.5 MB array (the cluster table's size), and
 *   - global memory, a 64 MB array (R-MAT-24's contribution vector),
 * both global cases served by L2.  The pull gather reads one random value
 * per in-edge, so the L2 rate bounds its non-hot gathers and the shared
 * rates bound what any on-chip table of hot values could serve.
 */
#include <cooperative_groups.h>

#include "gg_internal.h"

namespace cg = cooperative_groups;

namespace
{

constexpr int CL = 8;             // CTAs per cluster
constexpr int PER = 46 * 1024;    // values per CTA (184 KB of shared memory)
constexpr int K = CL * PER;       // values in a cluster's table
constexpr int THREADS = 1024;
constexpr int G = 4096;           // gathers per thread
constexpr uint32_t BIG = 16u << 20; // 64 MB of floats

__device__ __forceinline__ uint32_t mix(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
/* an index below n from a 32-bit hash (multiply-high, no division) */
__device__ __forceinline__ uint32_t pick(uint32_t x, uint32_t n) { return (uint32_t)(((uint64_t)x * n) >> 32); }

/* mode 0: values from the whole cluster's shared memory; 1: from the CTA's own */
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(THREADS, 1)
    k_gather_smem(const float *__restrict__ src, float *out, int mode)
{
    extern __shared__ float tab[];
    cg::cluster_group cl = cg::this_cluster();
    const uint32_t rank = cl.block_rank();
    for (int i = threadIdx.x; i < PER; i += THREADS) tab[i] = src[rank * PER + i];
    cl.sync();
    const uint32_t tid = blockIdx.x * THREADS + threadIdx.x;
    float acc = 0.f;
    if (mode == 0)
    {
#pragma unroll 8
        for (int j = 0; j < G; j++)
        {
            const uint32_t idx = pick(mix(tid * 0x9E3779B1u + j), K);
            const float *peer = cl.map_shared_rank(tab, idx / PER);
            acc += peer[idx % PER];
        }
    }
    else
    {
#pragma unroll 8
        for (int j = 0; j < G; j++) acc += tab[pick(mix(tid * 0x9E3779B1u + j), PER)];
    }
    cl.sync(); /* no CTA leaves while a peer may still read its table */
    out[tid] = acc;
}

__global__ void __launch_bounds__(THREADS, 1) k_gather_global(const float *__restrict__ src, uint32_t n, float *out)
{
    const uint32_t tid = blockIdx.x * THREADS + threadIdx.x;
    float acc = 0.f;
#pragma unroll 8
    for (int j = 0; j < G; j++) acc += __ldcg(src + pick(mix(tid * 0x9E3779B1u + j), n));
    out[tid] = acc;
}

struct Bufs
{
    float *big = nullptr, *out = nullptr;
    cudaEvent_t a = nullptr, b = nullptr;
    ~Bufs()
    {
        if (big) cudaFree(big);
        if (out) cudaFree(out);
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
};

} // namespace

extern "C" gg_status gg_gather_ceiling(gg_gather_rates *r, void *stream)
{
    if (!r) return gg_fail(GG_ERR_INVALID, "NULL argument");
    GgRange range("gg_gather_ceiling");
    memset(r, 0, sizeof(*r));
    cudaStream_t s = (cudaStream_t)stream;
    const size_t smem = (size_t)PER * sizeof(float);
    GG_CUDA(cudaFuncSetAttribute(k_gather_smem, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int clusters = 0;
    {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(CL * 64);
        cfg.blockDim = dim3(THREADS);
        cfg.dynamicSmemBytes = smem;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = CL;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        GG_CUDA(cudaOccupancyMaxActiveClusters(&clusters, k_gather_smem, &cfg));
    }
    if (clusters < 1) return gg_fail(GG_ERR_CUDA, "no 8-CTA cluster fits on this GPU");
    const int sblocks = clusters * CL, gblocks = gg_sm_count();
    const int maxb = sblocks > gblocks ? sblocks : gblocks;
    Bufs B;
    GG_CUDA(cudaMalloc(&B.big, (size_t)BIG * sizeof(float)));
    GG_CUDA(cudaMalloc(&B.out, (size_t)maxb * THREADS * sizeof(float)));
    GG_CUDA(cudaMemsetAsync(B.big, 0, (size_t)BIG * sizeof(float), s));
    GG_CUDA(cudaEventCreate(&B.a));
    GG_CUDA(cudaEventCreate(&B.b));
    double rate[4];
    for (int m = 0; m < 4; m++)
    {
        float best = 1e30f;
        for (int rep = 0; rep < 6; rep++)
        {
            GG_CUDA(cudaEventRecord(B.a, s));
            if (m < 2)
                k_gather_smem<<<sblocks, THREADS, smem, s>>>(B.big, B.out, m);
            else
                k_gather_global<<<gblocks, THREADS, 0, s>>>(B.big, m == 2 ? (uint32_t)K : BIG, B.out);
            GG_CUDA(cudaGetLastError());
            GG_CUDA(cudaEventRecord(B.b, s));
            GG_CHECK(gg_wait(s));
            float ms = 0.f;
            GG_CUDA(cudaEventElapsedTime(&ms, B.a, B.b));
            if (rep > 0 && ms < best) best = ms; /* the first launch warms up */
        }
        const double n = (double)(m < 2 ? sblocks : gblocks) * THREADS * G;
        rate[m] = n / (best * 1e-3) / 1e9;
    }
    r->cluster_smem_gps = rate[0];
    r->own_smem_gps = rate[1];
    r->l2_small_gps = rate[2];
    r->l2_large_gps = rate[3];
    r->clusters = (uint32_t)clusters;
    r->cluster_sms = (uint32_t)sblocks;
    return GG_OK;
}
