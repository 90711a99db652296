/*
 * gg_server: a device-resident query server (see include/gg_server.h).
 *
 * Two worker threads, each with its own handle on the graph and its own
 * CUDA stream: the PPR worker owns the caller's mapping, the BFS worker a
 * gg_graph_share view, so batched PageRank and BFS overlap on the GPU.
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

/* dst[k][v] = rank[v * stride + k] for k < K: 32x32 tiles transposed
 * through shared memory so reads (vertex rows) and writes (per-query
 * vectors) are both coalesced */
__global__ void k_extract_columns(const float *__restrict__ rank, uint32_t stride, uint32_t V, uint32_t K,
                                  float *const *__restrict__ dst)
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
            if (v < V && k < K) t[y][x] = rank[(size_t)v * stride + k];
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

} // namespace

struct gg_server
{
    gg_graph *g = nullptr;    /* PPR worker's handle (the caller's mapping) */
    gg_graph *view = nullptr; /* BFS worker's handle */
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
    std::thread t_ppr, t_bfs;

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
    void bfs_loop();
};

void gg_server::ppr_loop()
{
    cudaSetDevice(device);
    const size_t rb = ppr_bytes();
    for (;;)
    {
        std::vector<uint64_t> batch;
        std::vector<uint32_t> seed_off(1, 0), seeds;
        {
            std::unique_lock<std::mutex> lk(mu);
            cv_work.wait(lk, [&] { return stop || (!ppr_q.empty() && held + rb <= p.mem_budget_bytes); });
            if (stop) return;
            const size_t room = (size_t)((p.mem_budget_bytes - held) / rb);
            const size_t k = std::min({ppr_q.size(), (size_t)p.max_ppr_batch, room});
            const double t0 = now_s();
            for (size_t i = 0; i < k; i++)
            {
                const uint64_t t = ppr_q.front();
                ppr_q.pop_front();
                Query &q = qs[t];
                q.info.start_s = t0;
                q.info.batch_size = (uint32_t)k;
                q.bytes = rb;
                held += rb;
                seeds.insert(seeds.end(), q.seeds.begin(), q.seeds.end());
                seed_off.push_back((uint32_t)seeds.size());
                batch.push_back(t);
            }
        }
        const uint32_t K = (uint32_t)batch.size();
        gg_ppr_params pp{K, p.ppr_iterations, p.damp, p.ppr_storage, 0};
        gg_ppr_result res;
        gg_status st = gg_ppr(g, &pp, seed_off.data(), seeds.empty() ? nullptr : seeds.data(), nullptr, &res, nullptr);
        std::vector<void *> bufs(K, nullptr);
        if (st == GG_OK)
        {
            for (uint32_t i = 0; i < K && st == GG_OK; i++)
                if (!(bufs[i] = take_buffer(rb))) st = gg_fail(GG_ERR_NOMEM, "server: no device memory for a result");
        }
        if (st == GG_OK)
        {
            uint32_t stride = 0;
            const float *rank = gg_ppr_device_ranks(g, &stride);
            cudaStream_t s = gg_stream(g, nullptr);
            void *dptrs = nullptr;
            st = gg_work(g, 24, (size_t)K * sizeof(void *), &dptrs);
            if (st == GG_OK)
            {
                cudaError_t e = cudaMemcpyAsync(dptrs, bufs.data(), (size_t)K * sizeof(void *), cudaMemcpyHostToDevice, s);
                if (e == cudaSuccess)
                {
                    const uint32_t tiles = ((V + 31) / 32) * ((K + 31) / 32);
                    k_extract_columns<<<std::min<uint32_t>(tiles, (uint32_t)gg_sm_count() * 16), 256, 0, s>>>(
                        rank, stride, V, K, (float *const *)dptrs);
                    e = cudaGetLastError();
                }
                st = e == cudaSuccess ? gg_wait(s) : gg_cuda_fail(e, "server: result extraction");
            }
        }
        std::lock_guard<std::mutex> lk(mu);
        for (uint32_t i = 0; i < K; i++)
        {
            finish(batch[i], st, bufs[i]);
            if (st != GG_OK && bufs[i]) free_ppr.push_back(bufs[i]);
        }
        cv_done.notify_all();
        cv_work.notify_all();
    }
}

void gg_server::bfs_loop()
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
    gg_server *S = new gg_server();
    S->g = g;
    S->p = *p;
    S->V = g->V;
    S->device = g->device;
    gg_status st = gg_graph_share(g, &S->view);
    if (st != GG_OK)
    {
        delete S;
        return st;
    }
    S->t_ppr = std::thread(&gg_server::ppr_loop, S);
    S->t_bfs = std::thread(&gg_server::bfs_loop, S);
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
    S->t_bfs.join();
    cudaSetDevice(S->device);
    for (auto &kv : S->qs)
        if (kv.second.result) cudaFree(kv.second.result);
    for (void *b : S->free_ppr) cudaFree(b);
    for (void *b : S->free_bfs) cudaFree(b);
    gg_graph_unmap(S->view);
    delete S;
    return GG_OK;
}
