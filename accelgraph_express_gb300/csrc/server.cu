/*
 * gg_server: a device-resident query server (see include/gg_server.h).
 *
 * Worker threads, each with its own handle on the graph and its own CUDA
 * stream: the PPR worker owns the caller's mapping and runs one continuous
 * batch (slots admitted and retired at iteration boundaries), each BFS
 * worker a gg_graph_share view, so PageRank and several BFS overlap on the
 * GPU.
 * Queries wait in two FIFO queues; results live in device buffers recycled
 * through per-size free lists.  A worker admits work only while the results
 * held plus the new ones fit the memory budget; gg_server_take returns a
 * result's bytes to the budget.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "gg_internal.h"
#include "gg_server.h"

namespace {

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Query
{
    uint32_t kind = GG_QUERY_PPR;
    std::vector<uint32_t> seeds;
    uint32_t source = 0;
    gg_query_info info{};
    bool ready = false;
    void *result = nullptr; /* device: PPR V floats; BFS V parents then V distances */
    size_t bytes = 0;       /* budget charged while the query holds a result (or will) */
};

/* dst[i][v] = rank[v * stride + col[i]] for i < K: 32x32 tiles transposed
 * through shared memory so reads (vertex rows) and writes (per-query
 * vectors) are both coalesced */
__global__ void k_extract_columns(const float *__restrict__ rank, uint32_t stride, uint32_t V, uint32_t K,
                                  const uint32_t *__restrict__ col, float *const *__restrict__ dst)
{
    __shared__ float t[32][33];
    const uint32_t ntv = (V + 31) / 32, ntk = (K + 31) / 32;
    for (uint32_t b = blockIdx.x; b < ntv * ntk; b += gridDim.x)
    {
        const uint32_t v0 = (b / ntk) * 32, k0 = (b % ntk) * 32;
        const uint32_t x = threadIdx.x & 31;
        for (uint32_t y = threadIdx.x >> 5; y < 32; y += blockDim.x >> 5)
        {
            const uint32_t v = v0 + y, k = k0 + x;
            if (v < V && k < K) t[y][x] = rank[(size_t)v * stride + col[k]];
        }
        __syncthreads();
        for (uint32_t y = threadIdx.x >> 5; y < 32; y += blockDim.x >> 5)
        {
            const uint32_t k = k0 + y, v = v0 + x;
            if (v < V && k < K) dst[k][v] = t[x][y];
        }
        __syncthreads();
    }
}

/* seed_idx[v[i]] = value for i < n */
__global__ void k_set_u32(uint32_t *a, const uint32_t *__restrict__ v, uint32_t n, uint32_t value)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[v[i]] = value;
}

constexpr uint32_t SLOTS = 64;      /* vectors per row of the running batch */
constexpr uint32_t NO_SEED = 0xffffffffu;

struct Slot
{
    bool busy = false;
    uint64_t ticket = 0;
    uint32_t done = 0;               /* iterations run */
    std::vector<uint32_t> seeds;
};

} // namespace

struct gg_server
{
    gg_graph *g = nullptr;         /* PPR worker's handle (the caller's mapping) */
    std::vector<gg_graph *> views; /* one handle per BFS worker */
    gg_server_params p{};
    int device = 0;
    uint32_t V = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<uint64_t> ppr_q, bfs_q;
    std::unordered_map<uint64_t, Query> qs;
    uint64_t next_ticket = 1;
    uint64_t held = 0;
    bool stop = false;
    std::vector<void *> free_ppr, free_bfs;
    std::thread t_ppr;
    std::vector<std::thread> t_bfs;

    size_t ppr_bytes() const { return (size_t)V * 4; }
    size_t bfs_bytes() const { return (size_t)V * 8; }

    /* a result buffer of `bytes` (the free list of its size, else a fresh one) */
    void *take_buffer(size_t bytes)
    {
        {
            std::lock_guard<std::mutex> lk(mu);
            auto &fl = bytes == ppr_bytes() ? free_ppr : free_bfs;
            if (!fl.empty())
            {
                void *b = fl.back();
                fl.pop_back();
                return b;
            }
        }
        void *b = nullptr;
        if (cudaMalloc(&b, bytes) != cudaSuccess)
        {
            cudaGetLastError();
            return nullptr;
        }
        return b;
    }

    /* publish a finished query (called with mu held) */
    void finish(uint64_t t, gg_status st, void *buf)
    {
        Query &q = qs[t];
        q.info.status = (uint32_t)st;
        q.info.done_s = now_s();
        q.result = st == GG_OK ? buf : nullptr;
        if (st != GG_OK)
        {
            held -= q.bytes;
            q.bytes = 0;
        }
        q.ready = true;
    }

    void ppr_loop();
    void bfs_loop(gg_graph *view);
};

/*
 * Continuous batching: the PPR worker keeps one running batch of up to 64
 * vector slots over the graph and advances every busy slot by one
 * iteration per round (one gather over the first 16, 32 or 64 slots, as
 * many as the busy ones need).  Between rounds it admits waiting queries
 * into free slots (lowest first, while the memory budget allows) and
 * retires the slots that have run all their iterations: in its last round
 * a slot writes its ranks to the rank rows and stores zero contributions,
 * so its columns are clean for the next query (a column left outside the
 * rounds' range is cleaned by one more covering round).  A query's vector
 * never reads another slot's values, sums in the same order whatever runs
 * beside it, and so equals the vector gg_ppr computes for it alone.
 */
void gg_server::ppr_loop()
{
    cudaSetDevice(device);
    const size_t rb = ppr_bytes();
    const int bf16 = p.ppr_storage == GG_STORE_BF16;
    cudaStream_t s = gg_stream(g, nullptr);
    void *cb[2] = {nullptr, nullptr}, *rank = nullptr, *seed_idx = nullptr, *d_seedv = nullptr, *d_tab = nullptr,
         *d_list = nullptr;
    float *tile_slots = nullptr;
    gg_status setup = gg_ppr_round_prepare(g, SLOTS, bf16, &cb[0], &cb[1], &tile_slots, s);
    if (setup == GG_OK) setup = gg_work(g, 22, (size_t)V * SLOTS * sizeof(float), &rank);
    if (setup == GG_OK) setup = gg_work(g, 21, (size_t)V * 4 + 16, &seed_idx);
    if (setup == GG_OK && cudaMemsetAsync(seed_idx, 0xff, (size_t)V * 4, s) != cudaSuccess)
        setup = gg_cuda_fail(cudaGetLastError(), "server: seed index");
    if (setup == GG_OK) setup = gg_wait(s);
    Slot slot[SLOTS];
    uint32_t parity = 0;
    uint64_t clean_next = 0; /* columns freed last round: covered once more */
    std::vector<uint32_t> prev_verts;
    const uint32_t cap = std::min<uint32_t>(p.max_ppr_batch, SLOTS);
    for (;;)
    {
        uint64_t fresh = 0, busy = 0;
        {
            std::unique_lock<std::mutex> lk(mu);
            auto any_busy = [&] {
                for (uint32_t k = 0; k < SLOTS; k++)
                    if (slot[k].busy) return true;
                return false;
            };
            cv_work.wait(lk, [&] {
                return stop || any_busy() || (!ppr_q.empty() && held + rb <= p.mem_budget_bytes);
            });
            if (stop) return;
            const double t0 = now_s();
            for (uint32_t k = 0; k < cap && !ppr_q.empty() && held + rb <= p.mem_budget_bytes; k++)
            {
                if (slot[k].busy) continue;
                const uint64_t t = ppr_q.front();
                ppr_q.pop_front();
                Query &q = qs[t];
                q.info.start_s = t0;
                q.bytes = rb;
                held += rb;
                if (setup != GG_OK)
                {
                    finish(t, setup, nullptr);
                    continue;
                }
                slot[k].busy = true;
                slot[k].ticket = t;
                slot[k].done = 0;
                slot[k].seeds = q.seeds;
                fresh |= 1ull << k;
            }
            uint32_t nbusy = 0;
            for (uint32_t k = 0; k < SLOTS; k++)
                if (slot[k].busy)
                {
                    busy |= 1ull << k;
                    nbusy++;
                }
            for (uint32_t k = 0; k < SLOTS; k++)
                if (fresh >> k & 1) qs[slot[k].ticket].info.batch_size = nbusy;
            if (setup != GG_OK)
            {
                cv_done.notify_all();
                cv_work.notify_all();
                continue;
            }
        }
        if (!busy && !clean_next) continue;
        /* the seed table of the busy slots: each seed vertex once, with the
         * initial rank and the teleport of every slot it seeds */
        std::vector<uint32_t> verts;
        std::unordered_map<uint32_t, uint32_t> index;
        for (uint32_t k = 0; k < SLOTS; k++)
            if (busy >> k & 1)
                for (uint32_t v : slot[k].seeds)
                    if (index.emplace(v, (uint32_t)verts.size()).second) verts.push_back(v);
        const uint32_t nv = (uint32_t)verts.size();
        std::vector<double> share((size_t)nv * SLOTS, 0.0);
        for (uint32_t k = 0; k < SLOTS; k++)
            if (busy >> k & 1)
                for (uint32_t v : slot[k].seeds) share[(size_t)index[v] * SLOTS + k] += 1.0 / (double)slot[k].seeds.size();
        std::vector<float> tab((size_t)nv * SLOTS * 2);
        for (size_t i = 0; i < share.size(); i++)
        {
            tab[i] = (float)share[i];
            tab[share.size() + i] = (float)((1.0 - (double)p.damp) * share[i]);
        }
        uint64_t last = 0;
        for (uint32_t k = 0; k < SLOTS; k++)
            if ((busy >> k & 1) && slot[k].done + 1 >= p.ppr_iterations) last |= 1ull << k;
        const uint64_t cover = busy | clean_next;
        const uint32_t top = cover ? 64 - (uint32_t)__builtin_clzll(cover) : 1;
        gg_ppr_round_args r;
        r.kp = top <= 16 ? 16 : top <= 32 ? 32 : 64;
        r.bf16 = bf16;
        r.cin = cb[parity];
        r.cout = cb[parity ^ 1];
        r.rank = (float *)rank;
        r.rank_mask = last;
        r.zero_mask = last;
        r.seed_idx = (const uint32_t *)seed_idx;
        r.slots = tile_slots;
        r.damp = p.damp;
        gg_status st = GG_OK;
        /* finished slots' results: one buffer each */
        std::vector<uint32_t> done_cols;
        std::vector<void *> bufs;
        for (uint32_t k = 0; k < SLOTS; k++)
            if (last >> k & 1)
            {
                void *b = take_buffer(rb);
                if (!b) st = gg_fail(GG_ERR_NOMEM, "server: no device memory for a result");
                done_cols.push_back(k);
                bufs.push_back(b);
            }
        const uint32_t nd = (uint32_t)done_cols.size();
        const size_t list_words = prev_verts.size() + (size_t)nd + 2 * (size_t)nd + 4;
        if (st == GG_OK) st = gg_work(g, 19, ((size_t)nv + 1) * 4, &d_seedv);
        if (st == GG_OK) st = gg_work(g, 20, (tab.size() + 4) * sizeof(float), &d_tab);
        if (st == GG_OK) st = gg_work(g, 24, list_words * 8, &d_list);
        if (st == GG_OK)
        {
            cudaError_t e = cudaSuccess;
            uint32_t *d_prev = (uint32_t *)d_list;
            uint32_t *d_cols = d_prev + prev_verts.size();
            float **d_dst = (float **)((char *)d_list + ((prev_verts.size() + nd + 1) / 2) * 8);
            if (!prev_verts.empty())
            {
                e = cudaMemcpyAsync(d_prev, prev_verts.data(), prev_verts.size() * 4, cudaMemcpyHostToDevice, s);
                if (e == cudaSuccess)
                    k_set_u32<<<64, 256, 0, s>>>((uint32_t *)seed_idx, d_prev, (uint32_t)prev_verts.size(), NO_SEED);
            }
            if (e == cudaSuccess && nv)
                e = cudaMemcpyAsync(d_seedv, verts.data(), (size_t)nv * 4, cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess && nv)
                e = cudaMemcpyAsync(d_tab, tab.data(), tab.size() * sizeof(float), cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess) e = cudaGetLastError();
            st = e == cudaSuccess ? GG_OK : gg_cuda_fail(e, "server: seed table");
            if (st == GG_OK)
                st = gg_ppr_round_seed(g, SLOTS, bf16, cb[parity], (const uint32_t *)d_seedv, nv, (const float *)d_tab,
                                       (uint32_t *)seed_idx, fresh, s);
            r.tele = (const float *)d_tab + (size_t)nv * SLOTS;
            if (st == GG_OK) st = gg_ppr_round(g, r, s);
            if (st == GG_OK && nd)
            {
                e = cudaMemcpyAsync(d_cols, done_cols.data(), (size_t)nd * 4, cudaMemcpyHostToDevice, s);
                if (e == cudaSuccess)
                    e = cudaMemcpyAsync(d_dst, bufs.data(), (size_t)nd * sizeof(void *), cudaMemcpyHostToDevice, s);
                if (e == cudaSuccess)
                {
                    const uint32_t tiles = ((V + 31) / 32) * ((nd + 31) / 32);
                    k_extract_columns<<<std::min<uint32_t>(tiles, (uint32_t)gg_sm_count() * 16), 256, 0, s>>>(
                        (const float *)rank, SLOTS, V, nd, d_cols, (float *const *)d_dst);
                    e = cudaGetLastError();
                }
                if (e != cudaSuccess) st = gg_cuda_fail(e, "server: result extraction");
            }
            if (st == GG_OK) st = gg_wait(s);
        }
        parity ^= 1;
        prev_verts = verts;
        clean_next = last;
        std::lock_guard<std::mutex> lk(mu);
        uint32_t di = 0;
        for (uint32_t k = 0; k < SLOTS; k++)
        {
            if (!(busy >> k & 1)) continue;
            slot[k].done++;
            const bool fin = (last >> k & 1) != 0;
            if (st != GG_OK || fin)
            {
                void *b = fin ? bufs[di++] : nullptr;
                finish(slot[k].ticket, st, b);
                if (st != GG_OK && b) free_ppr.push_back(b);
                slot[k] = Slot();
            }
        }
        if (st != GG_OK)
        {
            /* a failed round leaves the batch state unknown: start clean */
            setup = gg_ppr_round_prepare(g, SLOTS, bf16, &cb[0], &cb[1], &tile_slots, s);
            if (setup == GG_OK && cudaMemsetAsync(seed_idx, 0xff, (size_t)V * 4, s) != cudaSuccess)
                setup = gg_cuda_fail(cudaGetLastError(), "server: seed index");
            if (setup == GG_OK) setup = gg_wait(s);
            prev_verts.clear();
            clean_next = 0;
            parity = 0;
        }
        cv_done.notify_all();
        cv_work.notify_all();
    }
}

void gg_server::bfs_loop(gg_graph *view)
{
    cudaSetDevice(device);
    const size_t rb = bfs_bytes();
    for (;;)
    {
        uint64_t t;
        uint32_t source;
        {
            std::unique_lock<std::mutex> lk(mu);
            cv_work.wait(lk, [&] { return stop || (!bfs_q.empty() && held + rb <= p.mem_budget_bytes); });
            if (stop) return;
            t = bfs_q.front();
            bfs_q.pop_front();
            Query &q = qs[t];
            q.info.start_s = now_s();
            q.bytes = rb;
            held += rb;
            source = q.source;
        }
        gg_bfs_params bp{GG_BFS_DO, source, 15, 18, 0};
        gg_bfs_result res;
        memset(&res, 0, sizeof(res));
        gg_status st = gg_bfs(view, &bp, nullptr, nullptr, &res, nullptr);
        void *buf = nullptr;
        if (st == GG_OK && !(buf = take_buffer(rb))) st = gg_fail(GG_ERR_NOMEM, "server: no device memory for a result");
        if (st == GG_OK)
        {
            const int32_t *par;
            const uint32_t *dist;
            st = gg_bfs_device_results(view, &par, &dist);
            if (st == GG_OK)
            {
                cudaStream_t s = gg_stream(view, nullptr);
                cudaError_t e = cudaMemcpyAsync(buf, par, (size_t)V * 4, cudaMemcpyDeviceToDevice, s);
                if (e == cudaSuccess)
                    e = cudaMemcpyAsync((char *)buf + (size_t)V * 4, dist, (size_t)V * 4, cudaMemcpyDeviceToDevice, s);
                st = e == cudaSuccess ? gg_wait(s) : gg_cuda_fail(e, "server: BFS result copy");
            }
        }
        std::lock_guard<std::mutex> lk(mu);
        Query &q = qs[t];
        q.info.bfs_levels = res.levels;
        q.info.bfs_reached = res.processed_nodes;
        finish(t, st, buf);
        if (st != GG_OK && buf) free_bfs.push_back(buf);
        cv_done.notify_all();
        cv_work.notify_all();
    }
}

extern "C" gg_status gg_server_start(gg_graph *g, const gg_server_params *p, gg_server **out)
{
    if (!out) return gg_fail(GG_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (!g || !p) return gg_fail(GG_ERR_INVALID, "NULL argument");
    if (p->max_ppr_batch < 1 || p->max_ppr_batch > 64) return gg_fail(GG_ERR_INVALID, "max_ppr_batch must be 1..64");
    if (p->ppr_iterations < 1) return gg_fail(GG_ERR_INVALID, "ppr_iterations must be at least 1");
    if (!g->in_off || !g->out_off) return gg_fail(GG_ERR_INVALID, "the server needs GG_MAP_IN|GG_MAP_OUT");
    if (p->mem_budget_bytes < (uint64_t)g->V * 8) return gg_fail(GG_ERR_INVALID, "mem_budget_bytes below one BFS result (8V)");
    if (p->bfs_workers > 16) return gg_fail(GG_ERR_INVALID, "bfs_workers must be 0..16");
    gg_server *S = new gg_server();
    S->g = g;
    S->p = *p;
    S->V = g->V;
    S->device = g->device;
    const uint32_t nb = p->bfs_workers ? p->bfs_workers : 2;
    for (uint32_t i = 0; i < nb; i++)
    {
        gg_graph *view = nullptr;
        gg_status st = gg_graph_share(g, &view);
        if (st != GG_OK)
        {
            for (gg_graph *v : S->views) gg_graph_unmap(v);
            delete S;
            return st;
        }
        S->views.push_back(view);
    }
    S->t_ppr = std::thread(&gg_server::ppr_loop, S);
    for (gg_graph *v : S->views) S->t_bfs.emplace_back(&gg_server::bfs_loop, S, v);
    *out = S;
    return GG_OK;
}

static gg_status submit(gg_server *S, Query &&q, uint64_t *ticket)
{
    q.info.kind = q.kind;
    q.info.submit_s = now_s();
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stop) return gg_fail(GG_ERR_INVALID, "server stopped");
    const uint64_t t = S->next_ticket++;
    const uint32_t kind = q.kind;
    S->qs.emplace(t, std::move(q));
    (kind == GG_QUERY_PPR ? S->ppr_q : S->bfs_q).push_back(t);
    if (ticket) *ticket = t;
    S->cv_work.notify_all();
    return GG_OK;
}

extern "C" gg_status gg_server_submit_ppr(gg_server *S, const uint32_t *seeds, uint32_t nseeds, uint64_t *ticket)
{
    if (!S || (nseeds && !seeds)) return gg_fail(GG_ERR_INVALID, "NULL argument");
    for (uint32_t i = 0; i < nseeds; i++)
        if (seeds[i] >= S->V) return gg_fail(GG_ERR_INVALID, "seed vertex out of range");
    Query q;
    q.kind = GG_QUERY_PPR;
    q.seeds.assign(seeds, seeds + nseeds);
    return submit(S, std::move(q), ticket);
}

extern "C" gg_status gg_server_submit_bfs(gg_server *S, uint32_t source, uint64_t *ticket)
{
    if (!S) return gg_fail(GG_ERR_INVALID, "NULL argument");
    if (source >= S->V) return gg_fail(GG_ERR_INVALID, "source out of range");
    Query q;
    q.kind = GG_QUERY_BFS;
    q.source = source;
    return submit(S, std::move(q), ticket);
}

extern "C" gg_status gg_server_take(gg_server *S, uint64_t ticket, uint32_t timeout_ms, gg_query_info *info,
                                    float *ppr, int32_t *parents, uint32_t *distances)
{
    if (!S) return gg_fail(GG_ERR_INVALID, "NULL argument");
    Query q;
    {
        std::unique_lock<std::mutex> lk(S->mu);
        auto it = S->qs.find(ticket);
        if (it == S->qs.end()) return gg_fail(GG_ERR_INVALID, "unknown ticket");
        auto done = [&] {
            auto i = S->qs.find(ticket);
            return i == S->qs.end() || i->second.ready;
        };
        if (!S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), done))
            return gg_fail(GG_ETIMEDOUT, "query not finished within the timeout");
        it = S->qs.find(ticket);
        if (it == S->qs.end()) return gg_fail(GG_ERR_INVALID, "query dropped by gg_server_stop");
        q = std::move(it->second);
        S->qs.erase(it);
    }
    if (info) *info = q.info;
    gg_status st = GG_OK;
    if (q.result)
    {
        cudaSetDevice(S->device);
        cudaError_t e = cudaSuccess;
        if (q.kind == GG_QUERY_PPR && ppr)
            e = cudaMemcpy(ppr, q.result, (size_t)S->V * 4, cudaMemcpyDeviceToHost);
        if (q.kind == GG_QUERY_BFS && parents && e == cudaSuccess)
            e = cudaMemcpy(parents, q.result, (size_t)S->V * 4, cudaMemcpyDeviceToHost);
        if (q.kind == GG_QUERY_BFS && distances && e == cudaSuccess)
            e = cudaMemcpy(distances, (char *)q.result + (size_t)S->V * 4, (size_t)S->V * 4, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) st = gg_cuda_fail(e, "server: result copy to host");
    }
    std::lock_guard<std::mutex> lk(S->mu);
    if (q.result) (q.kind == GG_QUERY_PPR ? S->free_ppr : S->free_bfs).push_back(q.result);
    S->held -= q.bytes;
    S->cv_work.notify_all();
    if (st != GG_OK) return st;
    return (gg_status)q.info.status;
}

extern "C" gg_status gg_server_stop(gg_server *S)
{
    if (!S) return GG_OK;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
        /* queries not started are dropped */
        for (uint64_t t : S->ppr_q) S->qs.erase(t);
        for (uint64_t t : S->bfs_q) S->qs.erase(t);
        S->ppr_q.clear();
        S->bfs_q.clear();
    }
    S->cv_work.notify_all();
    S->t_ppr.join();
    for (std::thread &t : S->t_bfs) t.join();
    cudaSetDevice(S->device);
    for (auto &kv : S->qs)
        if (kv.second.result) cudaFree(kv.second.result);
    for (void *b : S->free_ppr) cudaFree(b);
    for (void *b : S->free_bfs) cudaFree(b);
    for (gg_graph *v : S->views) gg_graph_unmap(v);
    delete S;
    return GG_OK;
}
