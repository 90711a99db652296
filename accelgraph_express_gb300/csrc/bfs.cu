/*
 * Breadth-first search on CSR (02_capi_graph/src/algorithms/capi/BFS.c:241-1110)
 * on one GPU.
 *
 * Device state: parents (int32, -outdeg = unvisited as in BFS.c:45-81),
 * distances (uint32), a visited bitmap, frontier queues and frontier
 * bitmaps.  Kernels:
 *   k_td  top-down step (BFS.c:688-750): one warp per frontier vertex, lanes
 *         over its out-edges, CAS claim of parents[u], warp-aggregated
 *         enqueue (ballot + popc + one atomic per warp), mf += -old parent
 *   k_bu  bottom-up step (BFS.c:752-803): one warp per 32-vertex bitmap word;
 *         each unvisited lane checks its first in-neighbours alone, longer
 *         lists are scanned by the whole warp 32 at a time with a ballot, so
 *         the parent is the first in-CSC neighbour in the frontier as in the
 *         reference; the warp owns its words of the next-frontier and visited
 *         bitmaps and writes them without atomics
 *   k_compact  bitmap -> queue (ballot/popc compaction)
 * The host drives the direction switch with the reference's uint32
 * arithmetic (alpha 15, beta 18, mu/mf/nf, BFS.c:555-650), reading three
 * counters after each step.
 */
#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include "gg_device.cuh"

namespace {

using namespace gg;

struct Counters
{
    uint32_t qlen;   /* next queue length */
    uint32_t mf;     /* top-down: sum of -parent of claimed vertices */
    uint32_t nf;     /* bottom-up: vertices found */
    uint32_t nheavy; /* top-down: frontier vertices deferred to k_td_heavy */
    unsigned long long edges;
};

constexpr int BU_SERIAL = 4;  /* in-neighbours a lane checks before the warp helps */

__global__ void k_bfs_init(const uint32_t *__restrict__ outdeg, int32_t *parents, uint32_t *dist, uint32_t *visited,
                           uint32_t V, uint32_t words)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
    {
        uint32_t d = outdeg[v];
        parents[v] = d ? -(int32_t)d : -1;
        dist[v] = 0u;
    }
    for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < words; w += gridDim.x * blockDim.x)
        visited[w] = 0u;
}

__global__ void k_bfs_source(int32_t *parents, uint32_t *visited, uint32_t *queue, uint32_t src)
{
    parents[src] = (int32_t)src;
    visited[src >> 5] |= 1u << (src & 31);
    queue[0] = src;
}

__device__ __forceinline__ bool bit_of(const uint32_t *bm, uint32_t v) { return (bm[v >> 5] >> (v & 31)) & 1u; }

/* top-down step from a queue; writes the next queue and, when nbm is set,
 * the next frontier bitmap */
/* claim out-neighbour u of v for the next level; returns whether this
 * thread won it (the reference's CAS, BFS.c:721-735) */
__device__ __forceinline__ bool td_claim(uint32_t u, uint32_t v, int32_t *parents, uint32_t *dist, uint32_t newdist,
                                         uint32_t *visited, uint32_t *nbm, uint32_t &mf)
{
    const int32_t p = parents[u];
    if (p < 0 && atomicCAS(&parents[u], p, (int32_t)v) == p)
    {
        mf += (uint32_t)(-p);
        dist[u] = newdist;
        atomicOr(&visited[u >> 5], 1u << (u & 31));
        if (nbm) atomicOr(&nbm[u >> 5], 1u << (u & 31));
        return true;
    }
    return false;
}

/* warp-aggregated append of the claimed vertices to the next queue */
__device__ __forceinline__ void td_enqueue(bool claimed, uint32_t u, uint32_t lane, uint32_t *nq, Counters *c)
{
    const uint32_t m = __ballot_sync(0xffffffffu, claimed);
    if (m)
    {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(&c->qlen, (uint32_t)__popc(m));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (claimed) nq[base + __popc(m & ((1u << lane) - 1u))] = u;
    }
}

/* frontier vertices with more out-edges than this go to k_td_heavy, at most
 * TD_MAX_HEAVY of them per step (further ones stay with their warp) */
#define TD_HEAVY 1024u
#define TD_MAX_HEAVY 4096u

__global__ void __launch_bounds__(256) k_td(const uint32_t *__restrict__ q, uint32_t qlen,
                                            const uint32_t *__restrict__ off, const uint32_t *__restrict__ adj,
                                            int32_t *parents, uint32_t *dist, uint32_t newdist, uint32_t *visited,
                                            uint32_t *nq, uint32_t *nbm, Counters *c, uint4 *heavy)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    uint32_t mf = 0;
    unsigned long long edges = 0;
    for (uint32_t i = warp; i < qlen; i += nwarps)
    {
        const uint32_t v = q[i];
        const uint32_t s = off[v], e = off[v + 1];
        if (lane == 0) edges += e - s;
        if (e - s > TD_HEAVY)
        {
            uint32_t slot = 0;
            if (lane == 0) slot = atomicAdd(&c->nheavy, 1u);
            slot = __shfl_sync(0xffffffffu, slot, 0);
            if (slot < TD_MAX_HEAVY)
            {
                if (lane == 0) heavy[slot] = make_uint4(v, s, e, 0u);
                continue;
            }
        }
        for (uint32_t b = s; b < e; b += 32)
        {
            const uint32_t j = b + lane;
            bool claimed = false;
            uint32_t u = 0;
            if (j < e)
            {
                u = adj[j];
                claimed = td_claim(u, v, parents, dist, newdist, visited, nbm, mf);
            }
            td_enqueue(claimed, u, lane, nq, c);
        }
    }
    mf = warp_sum(mf);
    edges = warp_sum(edges);
    if (lane == 0)
    {
        if (mf) atomicAdd(&c->mf, mf);
        if (edges) atomicAdd(&c->edges, edges);
    }
}

/* the deferred high-degree frontier vertices: their out-edges, concatenated,
 * are split evenly over the whole grid; every CTA scans the list's degrees
 * in shared memory and maps an edge index to its vertex by binary search */
__global__ void __launch_bounds__(256) k_td_heavy(const uint4 *__restrict__ heavy, const uint32_t *__restrict__ adj,
                                                  int32_t *parents, uint32_t *dist, uint32_t newdist,
                                                  uint32_t *visited, uint32_t *nq, uint32_t *nbm, Counters *c)
{
    __shared__ uint32_t pre[TD_MAX_HEAVY + 1];
    __shared__ uint32_t wsum[8];
    const uint32_t nh = min(c->nheavy, TD_MAX_HEAVY);
    if (nh == 0) return;
    const uint32_t tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    /* exclusive scan of the degrees: 16 consecutive entries per thread, then
     * the 256 thread totals through warp shuffles */
    constexpr uint32_t CH = TD_MAX_HEAVY / 256;
    uint32_t loc[CH], tot = 0;
#pragma unroll
    for (uint32_t k = 0; k < CH; k++)
    {
        const uint32_t i = tid * CH + k;
        loc[k] = i < nh ? heavy[i].z - heavy[i].y : 0u;
        tot += loc[k];
    }
    uint32_t incl = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += y;
    }
    if (lane == 31) wsum[w] = incl;
    __syncthreads();
    uint32_t wbase = 0;
    for (uint32_t k = 0; k < w; k++) wbase += wsum[k];
    uint32_t run = wbase + incl - tot;
#pragma unroll
    for (uint32_t k = 0; k < CH; k++)
    {
        pre[tid * CH + k] = run;
        run += loc[k];
    }
    if (tid == 255) pre[TD_MAX_HEAVY] = run;
    __syncthreads();
    const uint32_t H = pre[nh];
    uint32_t mf = 0;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x + (tid & ~31u); base < H; base += stride)
    {
        const uint32_t k = base + lane;
        bool claimed = false;
        uint32_t u = 0;
        if (k < H)
        {
            /* the last i with pre[i] <= k */
            uint32_t lo = 0, hi = nh - 1;
            while (lo < hi)
            {
                const uint32_t mid = (lo + hi + 1) >> 1;
                if (pre[mid] <= k)
                    lo = mid;
                else
                    hi = mid - 1;
            }
            const uint4 h = heavy[lo];
            u = adj[h.y + (k - pre[lo])];
            claimed = td_claim(u, h.x, parents, dist, newdist, visited, nbm, mf);
        }
        td_enqueue(claimed, u, lane, nq, c);
    }
    mf = warp_sum(mf);
    if (lane == 0 && mf) atomicAdd(&c->mf, mf);
}

/* bottom-up step: front -> next over in-edges */
__global__ void __launch_bounds__(256) k_bu(const uint32_t *__restrict__ off, const uint32_t *__restrict__ adj,
                                            int32_t *parents, uint32_t *dist, int write_dist, uint32_t newdist,
                                            const uint32_t *__restrict__ front, uint32_t *next, uint32_t *visited,
                                            uint32_t V, uint32_t words, Counters *c)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    uint32_t nf = 0;
    unsigned long long edges = 0;
    for (uint32_t w = warp; w < words; w += nwarps)
    {
        const uint32_t vis = visited[w];
        const uint32_t v = w * 32 + lane;
        const bool unvis = v < V && !((vis >> lane) & 1u);
        if (__ballot_sync(0xffffffffu, unvis) == 0u)
        {
            if (lane == 0) next[w] = 0u;
            continue;
        }
        bool found = false;
        uint32_t parent = 0, scanned = 0, rs = 0, re = 0;
        if (unvis)
        {
            const uint32_t s = off[v], e = off[v + 1];
            const uint32_t kend = min(e, s + BU_SERIAL);
            for (uint32_t j = s; j < kend; j++)
            {
                const uint32_t u = adj[j];
                scanned++;
                if (bit_of(front, u)) { found = true; parent = u; break; }
            }
            rs = kend;
            re = found ? kend : e;
        }
        uint32_t pending = __ballot_sync(0xffffffffu, unvis && !found && re > rs);
        while (pending)
        {
            const int ln = __ffs(pending) - 1;
            pending &= pending - 1;
            const uint32_t ws = __shfl_sync(0xffffffffu, rs, ln), we = __shfl_sync(0xffffffffu, re, ln);
            uint32_t cnt = 0, par = 0;
            bool hit_any = false;
            for (uint32_t b = ws; b < we; b += 32)
            {
                const uint32_t j = b + lane;
                uint32_t u = 0;
                bool hit = false;
                if (j < we)
                {
                    u = adj[j];
                    hit = bit_of(front, u);
                }
                const uint32_t m = __ballot_sync(0xffffffffu, hit);
                if (m)
                {
                    const int f = __ffs(m) - 1;
                    par = __shfl_sync(0xffffffffu, u, f);
                    cnt += (uint32_t)f + 1u;
                    hit_any = true;
                    break;
                }
                cnt += min(32u, we - b);
            }
            if (lane == (uint32_t)ln)
            {
                scanned += cnt;
                if (hit_any) { found = true; parent = par; }
            }
        }
        const uint32_t fm = __ballot_sync(0xffffffffu, found);
        if (found)
        {
            parents[v] = (int32_t)parent;
            if (write_dist) dist[v] = newdist;
        }
        if (lane == 0)
        {
            next[w] = fm;
            visited[w] = vis | fm;
            nf += (uint32_t)__popc(fm);
        }
        edges += scanned;
    }
    edges = warp_sum(edges);
    if (lane == 0)
    {
        if (nf) atomicAdd(&c->nf, nf);
        if (edges) atomicAdd(&c->edges, edges);
    }
}

/* frontier bitmap -> queue, one thread per word, warp-aggregated offsets */
__global__ void k_compact(const uint32_t *__restrict__ bm, uint32_t words, uint32_t *q, Counters *c)
{
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t w0 = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; w0 < words; w0 += gridDim.x * blockDim.x)
    {
        const uint32_t w = w0 + lane;
        uint32_t bits = w < words ? bm[w] : 0u;
        uint32_t n = (uint32_t)__popc(bits);
        uint32_t incl = n;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if ((int)lane >= o) incl += t;
        }
        uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
        uint32_t base = 0;
        if (lane == 0 && total) base = atomicAdd(&c->qlen, total);
        base = __shfl_sync(0xffffffffu, base, 0);
        uint32_t at = base + incl - n;
        while (bits)
        {
            const int b = __ffs(bits) - 1;
            bits &= bits - 1;
            q[at++] = w * 32 + (uint32_t)b;
        }
    }
}

__global__ void k_queue_to_bitmap(const uint32_t *__restrict__ q, uint32_t qlen, uint32_t *bm)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < qlen; i += gridDim.x * blockDim.x)
    {
        uint32_t v = q[i];
        atomicOr(&bm[v >> 5], 1u << (v & 31));
    }
}

int cap_blocks(uint64_t threads)
{
    uint64_t b = (threads + 255) / 256;
    uint64_t cap = (uint64_t)gg_sm_count() * 8;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

struct Bfs
{
    gg_graph *g;
    cudaStream_t s;
    uint32_t V, words;
    int32_t *parents;
    uint32_t *dist, *visited, *qa, *qb, *bma, *bmb;
    Counters *c;
    uint4 *heavy;      /* TD_MAX_HEAVY deferred frontier vertices (v, first, end) */
    Counters *h;       /* page-locked copy of *c */
    int profile;
    uint32_t launches = 0;
    std::vector<cudaEvent_t> evs;
    gg_bfs_result res{};
};

gg_status mark(Bfs &B)
{
    if (!B.profile) return GG_OK;
    cudaEvent_t e;
    GG_CHECK(gg_event_at(B.g, (uint32_t)B.evs.size(), &e));
    GG_CUDA(cudaEventRecord(e, B.s));
    B.evs.push_back(e);
    return GG_OK;
}

gg_status read_counters(Bfs &B)
{
    GG_CUDA(cudaMemcpyAsync(B.h, B.c, sizeof(Counters), cudaMemcpyDeviceToHost, B.s));
    GG_CHECK(gg_wait(B.s));
    B.res.edges_examined += B.h->edges;
    return GG_OK;
}

/* top-down from queue `q` (qlen) into queue `nq` (and bitmap `nbm`) */
gg_status td_step(Bfs &B, const uint32_t *q, uint32_t qlen, uint32_t *nq, uint32_t *nbm, uint32_t newdist)
{
    GG_CUDA(cudaMemsetAsync(B.c, 0, sizeof(Counters), B.s));
    if (nbm) GG_CUDA(cudaMemsetAsync(nbm, 0, (size_t)B.words * 4, B.s));
    GG_CHECK(mark(B));
    if (qlen)
    {
        k_td<<<cap_blocks((uint64_t)qlen * 32), 256, 0, B.s>>>(q, qlen, B.g->out_off, B.g->out_adj, B.parents, B.dist,
                                                                newdist, B.visited, nq, nbm, B.c, B.heavy);
        k_td_heavy<<<gg_sm_count() * 8, 256, 0, B.s>>>(B.heavy, B.g->out_adj, B.parents, B.dist, newdist, B.visited,
                                                       nq, nbm, B.c);
        B.launches += 2;
    }
    GG_CHECK(mark(B));
    B.res.top_down_steps++;
    GG_CUDA(cudaGetLastError());
    return read_counters(B);
}

gg_status bu_step(Bfs &B, const uint32_t *front, uint32_t *next, int write_dist, uint32_t newdist)
{
    GG_CUDA(cudaMemsetAsync(B.c, 0, sizeof(Counters), B.s));
    GG_CHECK(mark(B));
    k_bu<<<cap_blocks((uint64_t)B.words * 32), 256, 0, B.s>>>(B.g->in_off, B.g->in_adj, B.parents, B.dist, write_dist,
                                                              newdist, front, next, B.visited, B.V, B.words, B.c);
    GG_CHECK(mark(B));
    B.launches++;
    B.res.bottom_up_steps++;
    GG_CUDA(cudaGetLastError());
    return read_counters(B);
}

gg_status compact(Bfs &B, const uint32_t *bm, uint32_t *q, uint32_t *qlen)
{
    GG_CUDA(cudaMemsetAsync(B.c, 0, sizeof(Counters), B.s));
    k_compact<<<cap_blocks(B.words), 256, 0, B.s>>>(bm, B.words, q, B.c);
    B.launches++;
    GG_CUDA(cudaGetLastError());
    GG_CUDA(cudaMemcpyAsync(B.h, B.c, sizeof(Counters), cudaMemcpyDeviceToHost, B.s));
    GG_CHECK(gg_wait(B.s));
    *qlen = B.h->qlen;
    return GG_OK;
}

gg_status to_bitmap(Bfs &B, const uint32_t *q, uint32_t qlen, uint32_t *bm)
{
    GG_CUDA(cudaMemsetAsync(bm, 0, (size_t)B.words * 4, B.s));
    if (qlen) k_queue_to_bitmap<<<cap_blocks(qlen), 256, 0, B.s>>>(q, qlen, bm);
    B.launches++;
    GG_CUDA(cudaGetLastError());
    return GG_OK;
}

gg_status bfs_setup(Bfs &B, gg_graph *g, void *stream, int profile)
{
    B.g = g;
    B.s = gg_stream(g, stream);
    B.V = g->V;
    B.words = (g->V + 31) / 32;
    B.profile = profile;
    void *p;
    const size_t vb = ((size_t)B.V + 64) * 4, wb = ((size_t)B.words + 64) * 4;
    GG_CHECK(gg_work(g, 0, vb, &p)); B.parents = (int32_t *)p;
    GG_CHECK(gg_work(g, 1, vb, &p)); B.dist = (uint32_t *)p;
    GG_CHECK(gg_work(g, 2, vb, &p)); B.qa = (uint32_t *)p;
    GG_CHECK(gg_work(g, 3, vb, &p)); B.qb = (uint32_t *)p;
    GG_CHECK(gg_work(g, 4, wb, &p)); B.bma = (uint32_t *)p;
    GG_CHECK(gg_work(g, 5, wb, &p)); B.bmb = (uint32_t *)p;
    GG_CHECK(gg_work(g, 6, wb, &p)); B.visited = (uint32_t *)p;
    GG_CHECK(gg_work(g, 7, 256, &p)); B.c = (Counters *)p;
    GG_CHECK(gg_pinned(g, sizeof(Counters), &p)); B.h = (Counters *)p;
    GG_CHECK(gg_work(g, 8, (size_t)TD_MAX_HEAVY * sizeof(uint4), &p)); B.heavy = (uint4 *)p;
    return GG_OK;
}

} // namespace

extern "C" gg_status gg_bfs_device_results(const gg_graph *g, const int32_t **parents, const uint32_t **distances)
{
    if (!g || !g->work[0].ptr || !g->work[1].ptr) return gg_fail(GG_ERR_INVALID, "no BFS has run on this mapping");
    if (parents) *parents = (const int32_t *)g->work[0].ptr;
    if (distances) *distances = (const uint32_t *)g->work[1].ptr;
    return GG_OK;
}

extern "C" gg_status gg_bfs(gg_graph *g, const gg_bfs_params *p, int32_t *parents, uint32_t *distances,
                            gg_bfs_result *r, void *stream)
{
    if (!g || !p) return gg_fail(GG_ERR_INVALID, "NULL argument");
    if (p->mode > 4) return gg_fail(GG_ERR_INVALID, "unknown BFS mode");
    if (p->source >= g->V) return gg_fail(GG_ERR_INVALID, "source out of range");
    const bool need_out = p->mode != GG_BFS_PULL, need_in = p->mode == GG_BFS_PULL || p->mode == GG_BFS_DO ||
                                                           p->mode == GG_BFS_DO_BITMAP;
    if (need_out && !g->out_off) return gg_fail(GG_ERR_INVALID, "top-down BFS needs GG_MAP_OUT");
    if (need_in && !g->in_off) return gg_fail(GG_ERR_INVALID, "bottom-up BFS needs GG_MAP_IN");
    if (!g->out_deg) return gg_fail(GG_ERR_INVALID, "mapping has no out-degrees");

    Bfs B;
    GG_CHECK(bfs_setup(B, g, stream, p->profile));
    const uint32_t V = B.V, src = p->source;
    k_bfs_init<<<cap_blocks(V), 256, 0, B.s>>>(g->out_deg, B.parents, B.dist, B.visited, V, B.words);
    k_bfs_source<<<1, 1, 0, B.s>>>(B.parents, B.visited, B.qa, src);
    B.launches += 2;
    GG_CUDA(cudaGetLastError());

    uint32_t outdeg_src = 0;
    GG_CUDA(cudaMemcpyAsync(&outdeg_src, g->out_deg + src, 4, cudaMemcpyDeviceToHost, B.s));
    GG_CHECK(gg_wait(B.s));

    const uint32_t alpha = p->alpha ? p->alpha : 15, beta = p->beta ? p->beta : 18;
    uint32_t processed = 1; /* the reference counts the source (BFS.c:368, :474, :588, :881) */
    uint32_t level = 0;
    uint32_t *q = B.qa, *nq = B.qb, *bm = B.bma, *nbm = B.bmb;
    uint32_t qlen = 1;

    switch (p->mode)
    {
    case GG_BFS_PULL:
    {
        /* BFS.c:284-422: bottom-up every level, no distances (the FPGA does
         * not write them) */
        GG_CHECK(to_bitmap(B, q, 1, bm));
        uint32_t nf = 1;
        while (nf)
        {
            GG_CHECK(bu_step(B, bm, nbm, 0, level + 1));
            nf = B.h->nf;
            std::swap(bm, nbm);
            processed += nf;
            level++;
        }
        break;
    }
    case GG_BFS_PUSH:
    case GG_BFS_PUSH_BITMAP:
    {
        /* BFS.c:424-523 (queue) and :841-930 (bitmap frontier) */
        while (qlen)
        {
            GG_CHECK(td_step(B, q, qlen, nq, p->mode == GG_BFS_PUSH_BITMAP ? nbm : nullptr, level + 1));
            qlen = B.h->qlen;
            std::swap(q, nq);
            std::swap(bm, nbm);
            processed += qlen;
            level++;
        }
        break;
    }
    default:
    {
        /* BFS.c:525-686 and :932-1060: direction-optimised, uint32 accounting */
        uint32_t mu = g->E, mf = outdeg_src, nf = 0, nf_prev = 0;
        const uint32_t n = V;
        while (qlen)
        {
            if (mf > (mu / alpha))
            {
                GG_CHECK(to_bitmap(B, q, qlen, bm));
                nf = qlen;
                do
                {
                    nf_prev = nf;
                    GG_CHECK(bu_step(B, bm, nbm, 1, level + 1));
                    nf = B.h->nf;
                    std::swap(bm, nbm);
                    processed += nf;
                    level++;
                } while ((nf > nf_prev) || (nf > (n / beta)));
                GG_CHECK(compact(B, bm, q, &qlen));
                mf = 1;
            }
            else
            {
                mu -= mf;
                GG_CHECK(td_step(B, q, qlen, nq, nullptr, level + 1));
                mf = B.h->mf;
                qlen = B.h->qlen;
                std::swap(q, nq);
                processed += qlen;
                level++;
            }
        }
        break;
    }
    }

    B.res.processed_nodes = processed;
    B.res.levels = level;
    B.res.launches = B.launches;
    if (parents) GG_CUDA(cudaMemcpyAsync(parents, B.parents, (size_t)V * 4, cudaMemcpyDeviceToHost, B.s));
    if (distances) GG_CUDA(cudaMemcpyAsync(distances, B.dist, (size_t)V * 4, cudaMemcpyDeviceToHost, B.s));
    GG_CHECK(gg_wait(B.s));
    if (p->profile)
        for (size_t i = 0; i + 1 < B.evs.size(); i += 2) B.res.step_ms += gg_event_ms(B.evs[i], B.evs[i + 1]);
    if (r) *r = B.res;
    return GG_OK;
}

extern "C" gg_status gg_bfs_step_host(gg_graph *g, int direction, const uint32_t *frontier, uint32_t frontier_len,
                                      int frontier_is_bitmap, int32_t *parents, uint32_t *distances,
                                      uint32_t *next_queue, uint32_t *next_bitmap, uint32_t *next_len,
                                      uint32_t *counter, void *stream)
{
    if (!g || !parents || !distances) return gg_fail(GG_ERR_INVALID, "NULL argument");
    if (direction == 0 && !g->out_off) return gg_fail(GG_ERR_INVALID, "top-down step needs GG_MAP_OUT");
    if (direction == 1 && !g->in_off) return gg_fail(GG_ERR_INVALID, "bottom-up step needs GG_MAP_IN");
    if (direction == 1 && !frontier_is_bitmap) return gg_fail(GG_ERR_INVALID, "bottom-up step takes a bitmap frontier");
    Bfs B;
    GG_CHECK(bfs_setup(B, g, stream, 0));
    const uint32_t V = B.V, words = B.words;
    GG_CUDA(cudaMemcpyAsync(B.parents, parents, (size_t)V * 4, cudaMemcpyHostToDevice, B.s));
    GG_CUDA(cudaMemcpyAsync(B.dist, distances, (size_t)V * 4, cudaMemcpyHostToDevice, B.s));
    /* visited = parents >= 0 */
    std::vector<uint32_t> vis(words, 0u);
    for (uint32_t v = 0; v < V; v++)
        if (parents[v] >= 0) vis[v >> 5] |= 1u << (v & 31);
    GG_CUDA(cudaMemcpyAsync(B.visited, vis.data(), (size_t)words * 4, cudaMemcpyHostToDevice, B.s));
    uint32_t qlen = 0;
    if (frontier_is_bitmap)
        GG_CUDA(cudaMemcpyAsync(B.bma, frontier, (size_t)words * 4, cudaMemcpyHostToDevice, B.s));
    else
    {
        qlen = frontier_len;
        if (qlen) GG_CUDA(cudaMemcpyAsync(B.qa, frontier, (size_t)qlen * 4, cudaMemcpyHostToDevice, B.s));
    }
    /* all frontier vertices share one distance; the new level is that + 1 */
    uint32_t newdist = 0;
    {
        uint32_t any = 0xffffffffu;
        if (frontier_is_bitmap)
        {
            for (uint32_t w = 0; w < words && any == 0xffffffffu; w++)
                if (frontier[w]) any = w * 32 + (uint32_t)__builtin_ctz(frontier[w]);
        }
        else if (qlen)
            any = frontier[0];
        if (any != 0xffffffffu && any < V) newdist = distances[any] + 1;
    }
    uint32_t cnt = 0, nlen = 0;
    if (direction == 0)
    {
        if (frontier_is_bitmap) GG_CHECK(compact(B, B.bma, B.qa, &qlen));
        GG_CHECK(td_step(B, B.qa, qlen, B.qb, B.bmb, newdist));
        cnt = B.h->mf;
        nlen = B.h->qlen;
        if (next_queue && nlen) GG_CUDA(cudaMemcpyAsync(next_queue, B.qb, (size_t)nlen * 4, cudaMemcpyDeviceToHost, B.s));
    }
    else
    {
        GG_CHECK(bu_step(B, B.bma, B.bmb, 1, newdist));
        cnt = B.h->nf;
        nlen = B.h->nf;
        if (next_queue)
        {
            uint32_t ql = 0;
            GG_CHECK(compact(B, B.bmb, B.qb, &ql));
            if (ql) GG_CUDA(cudaMemcpyAsync(next_queue, B.qb, (size_t)ql * 4, cudaMemcpyDeviceToHost, B.s));
        }
    }
    if (next_bitmap) GG_CUDA(cudaMemcpyAsync(next_bitmap, B.bmb, (size_t)words * 4, cudaMemcpyDeviceToHost, B.s));
    GG_CUDA(cudaMemcpyAsync(parents, B.parents, (size_t)V * 4, cudaMemcpyDeviceToHost, B.s));
    GG_CUDA(cudaMemcpyAsync(distances, B.dist, (size_t)V * 4, cudaMemcpyDeviceToHost, B.s));
    GG_CHECK(gg_wait(B.s));
    if (next_len) *next_len = nlen;
    if (counter) *counter = cnt;
    return GG_OK;
}
