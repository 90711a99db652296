/*
 * Breadth-first search on CSR (02_capi_graph/src/algorithms/capi/BFS.c:241-1110)
 * on one GPU.
 *
 * Device state: parents (int32, -outdeg = unvisited as in BFS.c:45-81),
 * distances (uint32), a visited bitmap, frontier queues and frontier
 * bitmaps.  Kernels:
 *   k_td  top-down step (BFS.c:688-750): one warp per frontier vertex, lanes
 *         over its out-edges, CAS claim of parents[u], warp-aggregated
 *         enqueue (ballot + popc + one atomic per warp), mf += -old parent;
 *         vertices above the heavy threshold go to k_td_heavy, which spreads
 *         their edges over the whole grid
 *   k_bu  bottom-up step (BFS.c:752-803): one warp per 32-vertex bitmap word;
 *         each unvisited lane checks its first 4 in-neighbours alone, the
 *         lanes still searching then scan the rest of their lists together,
 *         32 candidates per round with a ballot, so the parent is the first
 *         in-CSC neighbour in the frontier as in the reference; the warp owns
 *         its words of the next-frontier and visited bitmaps and writes them
 *         without atomics
 *   k_bfs_init  parents, distances, the visited bitmap (vertices without
 *         in-edges start visited), the source, and the device loop's
 *         control block and first bitmap cleared, in one pass
 *   k_compact  bitmap -> queue (block-wide scan, one atomic per block pass)
 * Step counters are added and read once per block, not per warp: atomics
 * and loads of one address from every warp queue at one L2 slice.
 * The direction switch follows the reference's uint32 arithmetic (alpha 15,
 * beta 18, mu/mf/nf, BFS.c:555-650).  Without profiling, the
 * direction-optimised modes run the whole level loop in one cooperative
 * launch (k_bfs_do, grid barriers between steps); the other modes and
 * profiled searches drive the steps from the host, reading the step counters
 * after each one.
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

/* parents = -outdeg (-1 for no out-edges), distances 0, and the visited
 * bitmap.  A vertex without in-edges can never be reached, so when the CSC
 * is mapped its visited bit starts set: bottom-up steps then skip it without
 * reading its (empty) in-edge range, which changes no count.  A thread takes
 * four consecutive vertices with 16-byte accesses; eight threads make one
 * bitmap word, joined by shuffles.  The arrays are allocation-aligned. */
/* The same pass places the source (parent = itself, visited, queue[0]) and
 * clears `zero` words (the direction-optimised search's control block and
 * first frontier bitmap; may be null). */
__global__ void k_bfs_init(const uint32_t *__restrict__ outdeg, const uint32_t *__restrict__ in_off, int32_t *parents,
                           uint32_t *dist, uint32_t *visited, uint32_t V, uint32_t words, uint32_t src,
                           uint32_t *queue, uint32_t *zero_a, uint32_t zero_a_words, uint32_t *zero_b,
                           uint32_t zero_b_words)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t nq = (uint64_t)words * 8, stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t gtid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gtid == 0) queue[0] = src;
    for (uint64_t i = gtid; i < zero_a_words; i += stride) zero_a[i] = 0u;
    for (uint64_t i = gtid; i < zero_b_words; i += stride) zero_b[i] = 0u;
    const uint64_t nq32 = (nq + 31) & ~31ull; /* whole warps take part in the shuffles */
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nq32; t += stride)
    {
        const uint64_t v0 = t * 4;
        uint32_t bits = 0;
        if (v0 + 4 <= V)
        {
            const uint4 d = reinterpret_cast<const uint4 *>(outdeg)[t];
            int4 p4 = make_int4(d.x ? -(int32_t)d.x : -1, d.y ? -(int32_t)d.y : -1, d.z ? -(int32_t)d.z : -1,
                                d.w ? -(int32_t)d.w : -1);
            if (src - v0 < 4)
            {
                const int32_t self = (int32_t)src;
                switch ((uint32_t)(src - v0))
                {
                case 0: p4.x = self; break;
                case 1: p4.y = self; break;
                case 2: p4.z = self; break;
                default: p4.w = self; break;
                }
            }
            reinterpret_cast<int4 *>(parents)[t] = p4;
            reinterpret_cast<uint4 *>(dist)[t] = make_uint4(0u, 0u, 0u, 0u);
            if (in_off)
            {
                const uint4 a = reinterpret_cast<const uint4 *>(in_off)[t];
                const uint32_t b = in_off[v0 + 4];
                bits = (uint32_t)(a.x == a.y) | (uint32_t)(a.y == a.z) << 1 | (uint32_t)(a.z == a.w) << 2 |
                       (uint32_t)(a.w == b) << 3;
            }
        }
        else if (v0 < V)
        {
            for (uint32_t k = 0; v0 + k < V; k++)
            {
                const uint64_t v = v0 + k;
                const uint32_t d = outdeg[v];
                parents[v] = v == src ? (int32_t)src : (d ? -(int32_t)d : -1);
                dist[v] = 0u;
                if (in_off && in_off[v + 1] == in_off[v]) bits |= 1u << k;
            }
        }
        uint32_t m = bits << (4 * (lane & 7));
        m |= __shfl_xor_sync(0xffffffffu, m, 1);
        m |= __shfl_xor_sync(0xffffffffu, m, 2);
        m |= __shfl_xor_sync(0xffffffffu, m, 4);
        if ((t >> 3) == (uint64_t)(src >> 5)) m |= 1u << (src & 31);
        if ((lane & 7) == 0 && t < nq) visited[t >> 3] = m;
    }
}

__device__ __forceinline__ bool bit_of(const uint32_t *bm, uint32_t v) { return (bm[v >> 5] >> (v & 31)) & 1u; }

/* adds the block's per-thread values to one 32-bit and one 64-bit counter
 * with one atomic each (same-address atomics from every warp serialise at
 * one L2 slice); every thread of the block calls it */
__device__ __forceinline__ void block_flush(uint32_t *p32, uint32_t v32, unsigned long long *p64, unsigned long long v64)
{
    __shared__ uint32_t s32;
    __shared__ unsigned long long s64;
    if (threadIdx.x == 0)
    {
        s32 = 0u;
        s64 = 0ull;
    }
    __syncthreads();
    v32 = warp_sum(v32);
    v64 = warp_sum(v64);
    if ((threadIdx.x & 31) == 0)
    {
        if (v32) atomicAdd(&s32, v32);
        if (v64) atomicAdd(&s64, v64);
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
        if (s32) atomicAdd(p32, s32);
        if (s64 && p64) atomicAdd(p64, s64);
    }
}

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

/* frontier vertices with more out-edges than `heavy_thr` (64 by default,
 * the tuned value per mapping otherwise) go to k_td_heavy, at most
 * TD_MAX_HEAVY of them per step (further ones stay with their warp) */
#define TD_MAX_HEAVY 4096u

__device__ __forceinline__ void td_body(const uint32_t *q, uint32_t qlen,
                                        const uint32_t *__restrict__ off, const uint32_t *__restrict__ adj,
                                        int32_t *parents, uint32_t *dist, uint32_t newdist, uint32_t *visited,
                                        uint32_t *nq, uint32_t *nbm, Counters *c, uint4 *heavy, uint32_t heavy_thr)
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
        if (e - s > heavy_thr)
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
    block_flush(&c->mf, mf, &c->edges, edges);
}

/* the deferred high-degree frontier vertices: their out-edges, concatenated,
 * are split evenly over the whole grid; every CTA scans the list's degrees
 * in shared memory and maps an edge index to its vertex by binary search */
__device__ __forceinline__ void td_heavy_body(const uint4 *heavy, const uint32_t *__restrict__ adj,
                                              int32_t *parents, uint32_t *dist, uint32_t newdist,
                                              uint32_t *visited, uint32_t *nq, uint32_t *nbm, Counters *c)
{
    __shared__ uint32_t pre[TD_MAX_HEAVY + 1];
    __shared__ uint32_t wsum[8];
    __shared__ uint32_t s_nh;
    if (threadIdx.x == 0) s_nh = min(*(volatile uint32_t *)&c->nheavy, TD_MAX_HEAVY);
    __syncthreads();
    const uint32_t nh = s_nh;
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
    block_flush(&c->mf, mf, nullptr, 0ull);
}

/* bottom-up step: front -> next over in-edges; one warp per bitmap word
 * (the warp owns its words of `next` and `visited`) */
__device__ __forceinline__ void bu_body(const uint32_t *__restrict__ off, const uint32_t *__restrict__ adj,
                                        int32_t *parents, uint32_t *dist, int write_dist, uint32_t newdist,
                                        const uint32_t *front, uint32_t *next, uint32_t *visited,
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
            /* the candidates' ids, then their frontier bits, as independent
             * loads; the count stops at the first hit as a serial scan would */
            uint32_t u[BU_SERIAL];
            bool hit[BU_SERIAL];
#pragma unroll
            for (int k = 0; k < BU_SERIAL; k++) u[k] = s + k < kend ? adj[s + k] : 0u;
#pragma unroll
            for (int k = 0; k < BU_SERIAL; k++) hit[k] = s + k < kend && bit_of(front, u[k]);
#pragma unroll
            for (int k = BU_SERIAL - 1; k >= 0; k--)
                if (hit[k]) { found = true; parent = u[k]; scanned = (uint32_t)k + 1u; }
            if (!found) scanned = kend - s;
            rs = kend;
            re = found ? kend : e;
        }
        /* the lanes still searching scan the rest of their lists together:
         * their remaining candidates are concatenated in lane order and taken
         * 32 per round, each lane finding the owner of its item by a binary
         * search over the running totals; an owner's first frontier hit in
         * its own range is its parent (the first in CSC order, as before),
         * and lanes that found one drop out of the next round */
        uint32_t pending = __ballot_sync(0xffffffffu, unvis && !found && re > rs);
        while (pending)
        {
            const bool mine = (pending >> lane) & 1u;
            const uint32_t len = mine ? re - rs : 0u;
            uint32_t incl = len;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1)
            {
                const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= (uint32_t)o) incl += y;
            }
            const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
            const uint32_t excl = incl - len;
            /* owner of item `lane`: the number of lanes whose total is <= lane */
            uint32_t owner = 0;
#pragma unroll
            for (uint32_t step = 16; step >= 1; step >>= 1)
                if (__shfl_sync(0xffffffffu, incl, owner + step - 1) <= lane) owner += step;
            const uint32_t o_excl = __shfl_sync(0xffffffffu, excl, owner);
            const uint32_t o_rs = __shfl_sync(0xffffffffu, rs, owner);
            uint32_t u = 0;
            bool hit = false;
            if (lane < total)
            {
                u = adj[o_rs + (lane - o_excl)];
                hit = bit_of(front, u);
            }
            const uint32_t hits = __ballot_sync(0xffffffffu, hit);
            /* this lane's items in the round are lanes [lo, hi) */
            const uint32_t lo = min(excl, 32u), hi = min(incl, 32u);
            const uint32_t range = (hi >= 32u ? 0xffffffffu : ((1u << hi) - 1u)) & ~(lo >= 32u ? 0xffffffffu : ((1u << lo) - 1u));
            const uint32_t mh = mine ? (hits & range) : 0u;
            const int fl = mh ? __ffs(mh) - 1 : (int)lane;
            const uint32_t par = __shfl_sync(0xffffffffu, u, fl);
            if (mine)
            {
                if (mh)
                {
                    found = true;
                    parent = par;
                    scanned += (uint32_t)fl - lo + 1u;
                }
                else
                {
                    scanned += hi - lo;
                    rs += hi - lo;
                }
            }
            pending = __ballot_sync(0xffffffffu, mine && !found && rs < re);
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
    block_flush(&c->nf, nf, &c->edges, edges);
}

/* frontier bitmap -> queue, one thread per word; offsets from a block-wide
 * scan and one atomic per block pass (blockDim.x a multiple of 32, at most
 * 1024).  With `clear` the words read are zeroed. */
__device__ __forceinline__ void compact_body(uint32_t *bm, uint32_t words, uint32_t *q, Counters *c, bool clear)
{
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_base;
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (uint32_t b0 = blockIdx.x * blockDim.x; b0 < words; b0 += gridDim.x * blockDim.x)
    {
        const uint32_t w = b0 + threadIdx.x;
        uint32_t bits = w < words ? bm[w] : 0u;
        if (clear && bits) bm[w] = 0u;
        const uint32_t n = (uint32_t)__popc(bits);
        uint32_t incl = n;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if ((int)lane >= o) incl += t;
        }
        if (lane == 31) s_warp[wid] = incl;
        __syncthreads();
        if (threadIdx.x == 0)
        {
            uint32_t run = 0;
            for (uint32_t k = 0; k < nwarps; k++)
            {
                const uint32_t x = s_warp[k];
                s_warp[k] = run;
                run += x;
            }
            s_base = run ? atomicAdd(&c->qlen, run) : 0u;
        }
        __syncthreads();
        uint32_t at = s_base + s_warp[wid] + incl - n;
        while (bits)
        {
            const int b = __ffs(bits) - 1;
            bits &= bits - 1;
            q[at++] = w * 32 + (uint32_t)b;
        }
        __syncthreads();
    }
}

__device__ __forceinline__ void q2bm_body(const uint32_t *q, uint32_t qlen, uint32_t *bm)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < qlen; i += gridDim.x * blockDim.x)
    {
        uint32_t v = q[i];
        atomicOr(&bm[v >> 5], 1u << (v & 31));
    }
}

__global__ void __launch_bounds__(256) k_td(const uint32_t *__restrict__ q, uint32_t qlen,
                                            const uint32_t *__restrict__ off, const uint32_t *__restrict__ adj,
                                            int32_t *parents, uint32_t *dist, uint32_t newdist, uint32_t *visited,
                                            uint32_t *nq, uint32_t *nbm, Counters *c, uint4 *heavy,
                                            uint32_t heavy_thr)
{
    td_body(q, qlen, off, adj, parents, dist, newdist, visited, nq, nbm, c, heavy, heavy_thr);
}
__global__ void __launch_bounds__(256) k_td_heavy(const uint4 *__restrict__ heavy, const uint32_t *__restrict__ adj,
                                                  int32_t *parents, uint32_t *dist, uint32_t newdist,
                                                  uint32_t *visited, uint32_t *nq, uint32_t *nbm, Counters *c)
{
    td_heavy_body(heavy, adj, parents, dist, newdist, visited, nq, nbm, c);
}
__global__ void __launch_bounds__(256) k_bu(const uint32_t *__restrict__ off, const uint32_t *__restrict__ adj,
                                            int32_t *parents, uint32_t *dist, int write_dist, uint32_t newdist,
                                            const uint32_t *__restrict__ front, uint32_t *next, uint32_t *visited,
                                            uint32_t V, uint32_t words, Counters *c)
{
    bu_body(off, adj, parents, dist, write_dist, newdist, front, next, visited, V, words, c);
}
__global__ void k_compact(const uint32_t *__restrict__ bm, uint32_t words, uint32_t *q, Counters *c)
{
    compact_body(const_cast<uint32_t *>(bm), words, q, c, false);
}
__global__ void k_queue_to_bitmap(const uint32_t *__restrict__ q, uint32_t qlen, uint32_t *bm)
{
    q2bm_body(q, qlen, bm);
}

/* ---- direction-optimised search in one cooperative launch ----
 *
 * The whole level loop of BFS.c:555-650 runs inside k_bfs_do: every thread
 * keeps the reference's uint32 control variables (mu, mf, nf, nf_prev, qlen)
 * in registers and updates them identically from the step counters after a
 * grid barrier, so the direction schedule, level count and edge count are
 * those of the host-driven loop without a host round trip per level.  Step
 * s accumulates into counter slot s % 3 and clears slot (s + 1) % 3, whose
 * last readers finished two barriers earlier. */

/* control block of one search (work slot 7, CTL_BYTES, zeroed before the
 * launch): three counter slots at 0, the results at 256, the barrier's
 * root counter at 512, and per group of blocks an arrival counter at
 * 1024 + 128 g and a release word at 4096 + 128 g -- separate 128-byte
 * lines, so the spinning blocks of one group do not queue behind the
 * arrivals or the other groups at one L2 slice */
constexpr size_t CTL_BYTES = 8192;

struct DoOut
{
    uint32_t processed, levels, td, bu;
    unsigned long long edges;
    uint32_t err, pad;
};

struct DoArgs
{
    const uint32_t *out_off, *out_adj, *in_off, *in_adj, *out_deg;
    int32_t *parents;
    uint32_t *dist, *visited, *q[2], *bm[2];
    Counters *c;  /* three slots */
    uint4 *heavy;
    char *ctl;
    unsigned long long bar_limit_ns; /* device-side wait limit of the grid barrier */
    uint32_t V, words, E, src, alpha, beta, heavy_thr;
};

/* the grid barrier (gg_device.cuh) over the control block, failures
 * recorded in DoOut::err */
__device__ __forceinline__ bool grid_barrier(char *ctl, unsigned long long limit_ns, unsigned int &gen)
{
    return gg::grid_barrier(ctl, &((DoOut *)(ctl + 256))->err, limit_ns, gen);
}

/* one read of a counter slot per block, shared with its threads */
__device__ __forceinline__ Counters read_counters_block(const Counters *c)
{
    __shared__ Counters s_c;
    if (threadIdx.x == 0)
    {
        const volatile Counters *v = c;
        s_c.qlen = v->qlen;
        s_c.mf = v->mf;
        s_c.nf = v->nf;
        s_c.nheavy = v->nheavy;
        s_c.edges = v->edges;
    }
    __syncthreads();
    const Counters r = s_c;
    __syncthreads();
    return r;
}

__device__ __forceinline__ void clear_slot(Counters *c)
{
    if (blockIdx.x == 0 && threadIdx.x == 0)
    {
        c->qlen = 0u;
        c->mf = 0u;
        c->nf = 0u;
        c->nheavy = 0u;
        c->edges = 0ull;
    }
}

__global__ void __launch_bounds__(256, 6) k_bfs_do(DoArgs a)
{
    __shared__ uint32_t s_mf;
    unsigned int gen = 0;
    const uint32_t n = a.V;
    if (threadIdx.x == 0) s_mf = a.out_deg[a.src];
    __syncthreads();
    uint32_t mu = a.E, mf = s_mf, nf = 0, nf_prev = 0, qlen = 1;
    uint32_t processed = 1, level = 0, td = 0, bu = 0, qcur = 0, bcur = 0, s = 0;
    unsigned long long edges = 0;
    bool ok = true;
    while (qlen && ok)
    {
        if (level > n + 1)
        {
            ok = false;
            break;
        }
        if (mf > (mu / a.alpha))
        {
            /* queue -> bitmap (bm[bcur] is clear: the host cleared it and
             * every compaction clears what it reads) */
            q2bm_body(a.q[qcur], qlen, a.bm[bcur]);
            if (!(ok = grid_barrier(a.ctl, a.bar_limit_ns, gen))) break;
            nf = qlen;
            do
            {
                nf_prev = nf;
                Counters *cs = a.c + s % 3;
                clear_slot(a.c + (s + 1) % 3);
                bu_body(a.in_off, a.in_adj, a.parents, a.dist, 1, level + 1, a.bm[bcur], a.bm[bcur ^ 1], a.visited,
                        a.V, a.words, cs);
                if (!(ok = grid_barrier(a.ctl, a.bar_limit_ns, gen))) break;
                const Counters k = read_counters_block(cs);
                nf = k.nf;
                edges += k.edges;
                bu++;
                bcur ^= 1;
                processed += nf;
                level++;
                s++;
            } while (((nf > nf_prev) || (nf > (n / a.beta))) && level <= n + 1);
            if (!ok) break;
            Counters *cs = a.c + s % 3;
            clear_slot(a.c + (s + 1) % 3);
            compact_body(a.bm[bcur], a.words, a.q[qcur], cs, true);
            if (!(ok = grid_barrier(a.ctl, a.bar_limit_ns, gen))) break;
            qlen = read_counters_block(cs).qlen;
            s++;
            mf = 1;
        }
        else
        {
            mu -= mf;
            Counters *cs = a.c + s % 3;
            clear_slot(a.c + (s + 1) % 3);
            td_body(a.q[qcur], qlen, a.out_off, a.out_adj, a.parents, a.dist, level + 1, a.visited, a.q[qcur ^ 1],
                    nullptr, cs, a.heavy, a.heavy_thr);
            if (!(ok = grid_barrier(a.ctl, a.bar_limit_ns, gen))) break;
            /* the deferred high-degree vertices, when there are any (every
             * block reads the same final count, so all skip together) */
            if (read_counters_block(cs).nheavy)
            {
                td_heavy_body(a.heavy, a.out_adj, a.parents, a.dist, level + 1, a.visited, a.q[qcur ^ 1], nullptr,
                              cs);
                if (!(ok = grid_barrier(a.ctl, a.bar_limit_ns, gen))) break;
            }
            const Counters k = read_counters_block(cs);
            mf = k.mf;
            qlen = k.qlen;
            edges += k.edges;
            td++;
            qcur ^= 1;
            processed += qlen;
            level++;
            s++;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0)
    {
        DoOut *out = (DoOut *)(a.ctl + 256);
        out->processed = processed;
        out->levels = level;
        out->td = td;
        out->bu = bu;
        out->edges = edges;
        if (!ok) atomicExch(&out->err, 1u);
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
                                                                newdist, B.visited, nq, nbm, B.c, B.heavy,
                                                                B.g->bfs_heavy);
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
    GG_CHECK(gg_work(g, 7, CTL_BYTES, &p)); B.c = (Counters *)p;
    GG_CHECK(gg_pinned(g, 256, &p)); B.h = (Counters *)p;
    static_assert(3 * sizeof(Counters) <= 256 && sizeof(DoOut) <= 256 && GG_BAR_BYTES <= CTL_BYTES,
                  "control layout");
    GG_CHECK(gg_work(g, 8, (size_t)TD_MAX_HEAVY * sizeof(uint4), &p)); B.heavy = (uint4 *)p;
    return GG_OK;
}

/* BFS.c:525-686 / :932-1060 as one cooperative launch of k_bfs_do; the
 * control block (three counter slots, the barrier, the results) lives in
 * work slot 7 and is read back once */
gg_status do_search(Bfs &B, const gg_bfs_params *p)
{
    gg_graph *g = B.g;
    char *ctl = (char *)B.c;
    /* the control block and the first bitmap were cleared by k_bfs_init */
    DoArgs a{};
    a.out_off = g->out_off;
    a.out_adj = g->out_adj;
    a.in_off = g->in_off;
    a.in_adj = g->in_adj;
    a.out_deg = g->out_deg;
    a.parents = B.parents;
    a.dist = B.dist;
    a.visited = B.visited;
    a.q[0] = B.qa;
    a.q[1] = B.qb;
    a.bm[0] = B.bma;
    a.bm[1] = B.bmb;
    a.c = (Counters *)ctl;
    a.heavy = B.heavy;
    a.ctl = ctl;
    a.bar_limit_ns = gg_barrier_limit_ns();
    a.heavy_thr = g->bfs_heavy;
    a.V = B.V;
    a.words = B.words;
    a.E = g->E;
    a.src = p->source;
    a.alpha = p->alpha ? p->alpha : 15;
    a.beta = p->beta ? p->beta : 18;
    int per_sm = gg_occupancy((const void *)k_bfs_do, 256, 0);
    if (per_sm < 1) return gg_fail(GG_ERR_CUDA, "k_bfs_do cannot be resident");
    if (per_sm > 8) per_sm = 8;
    void *args[] = {&a};
    GG_CUDA(cudaLaunchCooperativeKernel((const void *)k_bfs_do, dim3(gg_sm_count() * per_sm), dim3(256), args, 0, B.s));
    B.launches++;
    DoOut *h = (DoOut *)((char *)B.h + 64);
    GG_CUDA(cudaMemcpyAsync(h, ctl + 256, sizeof(DoOut), cudaMemcpyDeviceToHost, B.s));
    GG_CHECK(gg_wait(B.s));
    if (h->err) return gg_fail(GG_ERR_KERNEL, "BFS grid barrier timed out");
    B.res.processed_nodes = h->processed;
    B.res.levels = h->levels;
    B.res.top_down_steps = h->td;
    B.res.bottom_up_steps = h->bu;
    B.res.edges_examined = h->edges;
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
    GgRange range("gg_bfs");
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
    gg_tune_lookup(g, B.s);
    const uint32_t V = B.V, src = p->source;
    const bool device_loop = (p->mode == GG_BFS_DO || p->mode == GG_BFS_DO_BITMAP) && !p->profile;
    /* the device loop's control block and first bitmap are cleared by the
     * same pass */
    k_bfs_init<<<cap_blocks((uint64_t)B.words * 8), 256, 0, B.s>>>(
        g->out_deg, g->in_off, B.parents, B.dist, B.visited, V, B.words, src, B.qa,
        device_loop ? (uint32_t *)B.c : nullptr, device_loop ? (uint32_t)(CTL_BYTES / 4) : 0u,
        device_loop ? B.bma : nullptr, device_loop ? B.words : 0u);
    B.launches++;
    GG_CUDA(cudaGetLastError());

    uint32_t outdeg_src = 0;
    if (!device_loop)
    {
        GG_CHECK(gg_wait(B.s)); /* bounded, before a copy to pageable memory */
        GG_CUDA(cudaMemcpyAsync(&outdeg_src, g->out_deg + src, 4, cudaMemcpyDeviceToHost, B.s));
        GG_CHECK(gg_wait(B.s));
    }

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
        if (device_loop)
        {
            GG_CHECK(do_search(B, p));
            processed = B.res.processed_nodes;
            level = B.res.levels;
            break;
        }
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
    if (parents) GG_CHECK(gg_copy_d2h(parents, B.parents, (size_t)V * 4, B.s));
    if (distances) GG_CHECK(gg_copy_d2h(distances, B.dist, (size_t)V * 4, B.s));
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
