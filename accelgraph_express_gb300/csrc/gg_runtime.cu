/*
 * gg_runtime core: device context, graph mapping, work buffers, bounded
 * waits.  This is the GPU replacement of the reference's CAPI layer
 * (02_capi_graph/src/capi_utils/capienv.c): mapGraphCSRToWED (:396-438)
 * becomes gg_graph_map, setupAFUGraphCSR (:30-55) gg_device_init, the
 * unbounded waitAFU poll (:111-172) a wait with a time limit, releaseAFU
 * (:299-303) gg_graph_unmap.
 */
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <omp.h>
#include <unistd.h>
#include <sys/mman.h>

#include <atomic>
#include <cmath>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "gg_internal.h"

namespace {

thread_local std::string t_last_error;
std::atomic<uint32_t> g_wait_timeout_ms{0};
int g_sm_count = 0;

uint32_t wait_timeout_ms()
{
    uint32_t v = g_wait_timeout_ms.load();
    if (v == 0)
    {
        const char *env = getenv("GG_WAIT_TIMEOUT_MS");
        v = env ? (uint32_t)strtoul(env, nullptr, 10) : 0;
        if (v == 0) v = 120000;
        g_wait_timeout_ms.store(v);
    }
    return v;
}

size_t align_up(size_t n, size_t a) { return (n + a - 1) / a * a; }

} // namespace

gg_status gg_fail(gg_status s, const std::string &msg)
{
    t_last_error = msg;
    return s;
}

gg_status gg_cuda_fail(cudaError_t e, const char *what)
{
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation)
        return gg_fail(GG_ERR_NOMEM, m);
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
        return gg_fail(GG_ERR_NO_DEVICE, m);
    return gg_fail(GG_ERR_CUDA, m);
}

extern "C" const char *gg_last_error(void) { return t_last_error.c_str(); }

extern "C" void gg_set_wait_timeout_ms(uint32_t ms) { g_wait_timeout_ms.store(ms ? ms : 120000); }

static std::atomic<unsigned long long> g_barrier_limit_ns{2000000000ull};

extern "C" void gg_set_barrier_limit_us(uint32_t us)
{
    g_barrier_limit_ns.store(us ? (unsigned long long)us * 1000ull : 2000000000ull);
}

unsigned long long gg_barrier_limit_ns() { return g_barrier_limit_ns.load(); }

int gg_sm_count() { return g_sm_count > 0 ? g_sm_count : 152; }

int gg_occupancy(const void *kernel, int threads, size_t smem)
{
    /* a host-side computation of a few microseconds, asked per launch by
     * the single-launch kernels: kept per (kernel, block, shared memory,
     * device) */
    struct Entry
    {
        const void *kernel;
        int threads;
        size_t smem;
        int device, bps;
    };
    static std::mutex mu;
    static std::vector<Entry> cache;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) cudaGetLastError();
    {
        std::lock_guard<std::mutex> lk(mu);
        for (const Entry &e : cache)
            if (e.kernel == kernel && e.threads == threads && e.smem == smem && e.device == dev) return e.bps;
    }
    int bps = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kernel, threads, smem) != cudaSuccess)
    {
        cudaGetLastError();
        return 0;
    }
    std::lock_guard<std::mutex> lk(mu);
    cache.push_back(Entry{kernel, threads, smem, dev, bps});
    return bps;
}

int gg_persistent_grid(const void *kernel, uint32_t ntiles, int ctas_per_sm)
{
    /* per (kernel, requested CTAs per SM): the resident CTAs per SM and the
     * carve-out that holds them; the carve-out is a kernel attribute, so it
     * is set again whenever a kernel is launched with another request than
     * the one last applied to it */
    struct Shape
    {
        const void *kernel;
        int ctas, bps, pct;
    };
    struct Applied
    {
        const void *kernel;
        int pct;
    };
    static std::mutex mu;
    static Shape shapes[128];
    static Applied applied[64];
    static int nshapes = 0, napplied = 0;
    int bps = 0, pct = 0;
    {
        std::lock_guard<std::mutex> lk(mu);
        int found = -1;
        for (int i = 0; i < nshapes; i++)
            if (shapes[i].kernel == kernel && shapes[i].ctas == ctas_per_sm) found = i;
        if (found >= 0)
        {
            bps = shapes[found].bps;
            pct = shapes[found].pct;
        }
        else
        {
            cudaError_t e = cudaSuccess;
            if (ctas_per_sm > 0)
            {
                /* carve-out: the smallest share of the SM's shared-memory
                 * capacity that holds ctas_per_sm CTAs (1 KB reserved each) */
                cudaFuncAttributes fa;
                int dev = 0, smem_sm = 0;
                e = cudaFuncGetAttributes(&fa, kernel);
                if (e == cudaSuccess) e = cudaGetDevice(&dev);
                if (e == cudaSuccess) e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
                if (e == cudaSuccess && smem_sm > 0)
                {
                    const double need = (double)ctas_per_sm * (double)(fa.sharedSizeBytes + 1024);
                    pct = (int)ceil(100.0 * need / (double)smem_sm);
                    pct = pct < 1 ? 1 : (pct > 100 ? 100 : pct);
                    e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
                }
            }
            if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kernel, GG_TILE_NT, 0);
            if (e != cudaSuccess || bps < 1)
            {
                cudaGetLastError();
                bps = 1;
                pct = 0;
            }
            if (ctas_per_sm > 0 && bps > ctas_per_sm) bps = ctas_per_sm;
            if (getenv("GG_DEBUG"))
                fprintf(stderr, "gg: kernel %p: %d CTAs of %d threads per SM (%s)\n", kernel, bps, GG_TILE_NT,
                        cudaGetErrorString(e));
            if (nshapes < 128) shapes[nshapes++] = Shape{kernel, ctas_per_sm, bps, pct};
        }
        /* the carve-out applied to this kernel last */
        if (pct > 0)
        {
            int a = -1;
            for (int i = 0; i < napplied; i++)
                if (applied[i].kernel == kernel) a = i;
            if (a < 0 && napplied < 64)
            {
                a = napplied++;
                applied[a] = Applied{kernel, 0};
            }
            if (a >= 0 && applied[a].pct != pct)
            {
                if (cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, pct) == cudaSuccess)
                    applied[a].pct = pct;
                else
                    cudaGetLastError();
            }
        }
    }
    const uint64_t need = ((uint64_t)ntiles + GG_TILE_WARPS - 1) / GG_TILE_WARPS;
    const uint64_t cap = (uint64_t)gg_sm_count() * (uint64_t)bps;
    const uint64_t g = need < cap ? need : cap;
    return (int)(g < 1 ? 1 : g);
}

float gg_float_ceil(double x)
{
    if (x != x) return (float)x;
    float f = (float)x;
    if ((double)f < x) f = nextafterf(f, INFINITY);
    return f;
}

float gg_float_floor(double x)
{
    if (x != x) return (float)x;
    float f = (float)x;
    if ((double)f > x) f = nextafterf(f, -INFINITY);
    return f;
}

extern "C" gg_status gg_device_init(int device)
{
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0)
        return gg_fail(GG_ERR_NO_DEVICE, std::string("no CUDA device: ") +
                                             (e != cudaSuccess ? cudaGetErrorString(e) : "count is 0"));
    if (device < 0 || device >= n)
        return gg_fail(GG_ERR_INVALID, "device index out of range");
    GG_CUDA(cudaSetDevice(device));
    GG_CUDA(cudaDeviceGetAttribute(&g_sm_count, cudaDevAttrMultiProcessorCount, device));
    return GG_OK;
}

/* ---- device memory ------------------------------------------------------
 * Blocks the library frees are kept for reuse.  A mapping made and dropped
 * on every call (the drop-in entry points on a host graph) would otherwise
 * pay cudaMalloc and cudaFree for each of its arrays every time, about 1 ms
 * per GB-sized array on this system.  A block enters the cache once the
 * device is idle, the same point cudaFree's implicit synchronisation waited
 * for, so no queued kernel can still read it when it is handed out again.
 * A request takes the smallest cached block of its device that is at least
 * as large and at most 1/8 larger.  The cache holds at most
 * GG_DEVICE_CACHE_MB (default 16384) MB; the oldest blocks leave first.  An
 * allocation that fails empties it and tries again, and
 * gg_device_cache_trim() empties it on request. */
namespace {
struct CachedBlock
{
    void *ptr;
    size_t bytes;
    int device;
    uint64_t seq;
};
std::mutex g_cache_mu;
std::vector<CachedBlock> g_cache;
struct LiveBlock
{
    size_t bytes;
    int device;
};
std::unordered_map<void *, LiveBlock> g_live; /* block -> its allocated size and device */
size_t g_cache_bytes = 0;
uint64_t g_cache_seq = 0;

size_t cache_limit()
{
    static const size_t v = [] {
        const char *e = getenv("GG_DEVICE_CACHE_MB");
        return (size_t)(e ? strtoull(e, nullptr, 10) : 16384ull) << 20;
    }();
    return v;
}

/* the block of the cache's oldest entry leaves it (lock held) */
void cache_evict_oldest()
{
    size_t k = 0;
    for (size_t i = 1; i < g_cache.size(); i++)
        if (g_cache[i].seq < g_cache[k].seq) k = i;
    int cur = 0;
    cudaGetDevice(&cur);
    if (g_cache[k].device != cur) cudaSetDevice(g_cache[k].device);
    cudaFree(g_cache[k].ptr);
    if (g_cache[k].device != cur) cudaSetDevice(cur);
    g_cache_bytes -= g_cache[k].bytes;
    g_cache[k] = g_cache.back();
    g_cache.pop_back();
}

/* a freed block into the cache (its device is idle), or back to CUDA */
void cache_put(void *p, size_t fallback_bytes)
{
    std::lock_guard<std::mutex> lock(g_cache_mu);
    size_t bytes = fallback_bytes;
    int dev = -1;
    auto it = g_live.find(p);
    if (it != g_live.end())
    {
        bytes = it->second.bytes;
        dev = it->second.device;
        g_live.erase(it);
    }
    const size_t limit = cache_limit();
    if (bytes > limit || dev < 0)
    {
        cudaFree(p);
        return;
    }
    while (!g_cache.empty() && g_cache_bytes + bytes > limit) cache_evict_oldest();
    g_cache.push_back(CachedBlock{p, bytes, dev, ++g_cache_seq});
    g_cache_bytes += bytes;
}

/* free a block; device_idle: the caller has synchronised the device since
 * the block was last used */
void dev_release(gg_graph *g, void *p, size_t bytes, bool device_idle)
{
    if (!p) return;
    g->mem_gen++;
    const size_t b = align_up(bytes ? bytes : 256, 256);
    g->device_bytes = g->device_bytes >= b ? g->device_bytes - b : 0;
    if (!device_idle && cudaDeviceSynchronize() != cudaSuccess)
    {
        /* the context is in error: hand the block back to CUDA as before */
        cudaGetLastError();
        std::lock_guard<std::mutex> lock(g_cache_mu);
        g_live.erase(p);
        cudaFree(p);
        return;
    }
    cache_put(p, b);
}
} // namespace

extern "C" void gg_device_cache_trim(void)
{
    std::lock_guard<std::mutex> lock(g_cache_mu);
    while (!g_cache.empty()) cache_evict_oldest();
}

extern "C" size_t gg_device_cache_bytes(void)
{
    std::lock_guard<std::mutex> lock(g_cache_mu);
    return g_cache_bytes;
}

gg_status gg_dev_alloc(gg_graph *g, void **p, size_t bytes)
{
    *p = nullptr;
    const size_t need = align_up(bytes ? bytes : 256, 256);
    int dev = 0;
    GG_CUDA(cudaGetDevice(&dev));
    {
        std::lock_guard<std::mutex> lock(g_cache_mu);
        size_t best = g_cache.size();
        for (size_t i = 0; i < g_cache.size(); i++)
        {
            const CachedBlock &c = g_cache[i];
            if (c.device != dev || c.bytes < need || c.bytes > need + need / 8) continue;
            if (best == g_cache.size() || c.bytes < g_cache[best].bytes) best = i;
        }
        if (best < g_cache.size())
        {
            *p = g_cache[best].ptr;
            g_live[*p] = LiveBlock{g_cache[best].bytes, dev};
            g_cache_bytes -= g_cache[best].bytes;
            g_cache[best] = g_cache.back();
            g_cache.pop_back();
            g->device_bytes += need;
            return GG_OK;
        }
    }
    cudaError_t e = cudaMalloc(p, need);
    if (e == cudaErrorMemoryAllocation)
    {
        cudaGetLastError();
        gg_device_cache_trim();
        e = cudaMalloc(p, need);
    }
    if (e != cudaSuccess)
    {
        *p = nullptr;
        return gg_cuda_fail(e, "cudaMalloc");
    }
    {
        std::lock_guard<std::mutex> lock(g_cache_mu);
        g_live[*p] = LiveBlock{need, dev};
    }
    g->device_bytes += need;
    return GG_OK;
}

void gg_dev_free(gg_graph *g, void *p, size_t bytes) { dev_release(g, p, bytes, false); }

gg_status gg_work(gg_graph *g, int slot, size_t bytes, void **out)
{
    gg_buf &b = g->work[slot];
    if (b.bytes < bytes)
    {
        if (b.ptr) gg_dev_free(g, b.ptr, b.bytes);
        b.ptr = nullptr;
        b.bytes = 0;
        GG_CHECK(gg_dev_alloc(g, &b.ptr, bytes));
        b.bytes = bytes;
    }
    *out = b.ptr;
    return GG_OK;
}

gg_status gg_pinned(gg_graph *g, size_t bytes, void **out)
{
    if (g->pinned_bytes < bytes)
    {
        if (g->pinned) cudaFreeHost(g->pinned);
        g->pinned = nullptr;
        g->pinned_bytes = 0;
        GG_CUDA(cudaHostAlloc(&g->pinned, bytes, cudaHostAllocDefault));
        g->pinned_bytes = bytes;
    }
    *out = g->pinned;
    return GG_OK;
}

cudaStream_t gg_stream(gg_graph *g, void *user_stream)
{
    return user_stream ? (cudaStream_t)user_stream : g->own_stream;
}

/* Bounded host wait on a recorded event. */
static gg_status wait_event(cudaEvent_t ev)
{
    cudaError_t e;
    const auto t0 = std::chrono::steady_clock::now();
    const uint32_t limit = wait_timeout_ms();
    for (;;)
    {
        e = cudaEventQuery(ev);
        if (e == cudaSuccess) break;
        if (e != cudaErrorNotReady) return gg_cuda_fail(e, "device work");
        const auto us =
            std::chrono::duration_cast<std::chrono::microseconds>(std::chrono::steady_clock::now() - t0).count();
        if ((uint64_t)us > (uint64_t)limit * 1000)
            return gg_fail(GG_ETIMEDOUT, "device work did not finish within the wait limit");
        /* spin through the first half millisecond (per-level BFS waits and
         * short calls end within it), then nap briefly between polls */
        if (us > 500) std::this_thread::sleep_for(std::chrono::microseconds(5));
    }
    return GG_OK;
}

gg_status gg_wait(cudaStream_t s)
{
    /* Bounded host wait: poll an event instead of blocking forever like the
     * reference's waitAFU loop.  One event per host thread and device is
     * kept (creating one per wait cost microseconds on every call); one that
     * no longer records (its context was reset) is made again. */
    constexpr int MAXDEV = 16;
    thread_local cudaEvent_t t_ev[MAXDEV] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAXDEV)
    {
        cudaGetLastError();
        cudaEvent_t ev;
        GG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        cudaError_t e = cudaEventRecord(ev, s);
        const gg_status st = e == cudaSuccess ? wait_event(ev) : gg_cuda_fail(e, "cudaEventRecord");
        cudaEventDestroy(ev);
        return st;
    }
    cudaEvent_t &ev = t_ev[dev];
    cudaError_t e = cudaErrorInvalidResourceHandle;
    if (ev) e = cudaEventRecord(ev, s);
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        ev = nullptr;
        GG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        e = cudaEventRecord(ev, s);
        if (e != cudaSuccess) return gg_cuda_fail(e, "cudaEventRecord");
    }
    return wait_event(ev);
}

/* ---- copies between HBM and pageable host memory -------------------------
 * Copies from pageable memory take one of three routes
 * (gg_set_host_copy_mode).  Measured on a GB300 with a Grace host, a 2.1 GB
 * pageable edge list built into a CSR (upload included) inside a
 * long-running process, each route timed on the same list: through two
 * page-locked 32 MB buffers, each filled by all host threads while the
 * other's DMA runs, 42-45 ms every time; the driver's own pageable copy, or
 * a kernel reading the source in place through the host's page tables
 * (cudaDevAttrPageableMemoryAccessUsesHostPageTables), 30-31 ms once the
 * buffer had been copied before, but 197-357 ms when the direct route was
 * the first to read that buffer; page-locking the source in place for one
 * DMA (cudaHostRegister) 133 ms.  A caller's graph is typically uploaded
 * once, so the staging, whose rate does not depend on the state of the
 * host pages, is the default.  Copies to pageable memory where the GPU uses
 * the host's page tables are the driver's copy (~190 GB/s once the pages
 * are resident: gg_host_dst_prepare makes them so), else go through the
 * staging buffers. */
namespace {
int g_host_pt_device = -1;
std::atomic<int> g_host_pt{-1};

/* the current device reads pageable memory through the host page tables */
bool host_page_tables()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
    {
        cudaGetLastError();
        return false;
    }
    int v = g_host_pt.load();
    if (v < 0 || g_host_pt_device != dev)
    {
        int a = 0;
        if (cudaDeviceGetAttribute(&a, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess)
        {
            cudaGetLastError();
            a = 0;
        }
        g_host_pt_device = dev;
        v = a ? 1 : 0;
        g_host_pt.store(v);
    }
    return v == 1;
}

/* one write per host page of [p, p + n), on all host threads: pages never
 * touched are faulted in here, in parallel, instead of one by one under the
 * DMA (64 MB of fresh pages: 3.4 ms as a DMA target, 0.5 + 0.45 ms touched
 * first); pages already resident cost one store each */
void touch_pages(void *p, size_t n)
{
    static const size_t pg = [] {
        const long v = sysconf(_SC_PAGESIZE);
        return v > 0 ? (size_t)v : (size_t)4096;
    }();
    volatile unsigned char *b = (volatile unsigned char *)p;
    const size_t pages = (n + pg - 1) / pg;
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < pages; i++) b[i * pg] = 0;
    if (n) b[n - 1] = 0;
}

__global__ void k_copy_from_host(const uint4 *__restrict__ src, uint4 *__restrict__ dst, size_t n16)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n16; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

constexpr size_t STAGE_BYTES = (size_t)32 << 20;
std::mutex g_stage_mu;
void *g_stage[2] = {nullptr, nullptr};
cudaEvent_t g_stage_ev[2] = {nullptr, nullptr};

void parallel_copy(void *to, const void *from, size_t n)
{
#pragma omp parallel
    {
        const size_t T = (size_t)omp_get_num_threads(), t = (size_t)omp_get_thread_num();
        const size_t a = n * t / T / 64 * 64, e = t + 1 == T ? n : n * (t + 1) / T / 64 * 64;
        if (e > a) memcpy((unsigned char *)to + a, (const unsigned char *)from + a, e - a);
    }
}

bool host_pinned(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess)
    {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}
} // namespace

static std::atomic<uint32_t> g_host_copy{0xffffffffu};

extern "C" void gg_set_host_copy_mode(uint32_t mode)
{
    g_host_copy.store(mode <= GG_HOST_COPY_DEVICE ? mode : GG_HOST_COPY_AUTO);
}

extern "C" uint32_t gg_host_copy_mode(void)
{
    uint32_t m = g_host_copy.load();
    if (m == 0xffffffffu)
    {
        const char *e = getenv("GG_HOST_COPY");
        m = GG_HOST_COPY_AUTO;
        if (e && !strcmp(e, "staged")) m = GG_HOST_COPY_STAGED;
        if (e && !strcmp(e, "driver")) m = GG_HOST_COPY_DRIVER;
        if (e && !strcmp(e, "device")) m = GG_HOST_COPY_DEVICE;
        g_host_copy.store(m);
    }
    return m;
}

gg_status gg_copy_h2d(void *dst, const void *src, size_t bytes, cudaStream_t s)
{
    uint32_t mode = gg_host_copy_mode();
    if (mode == GG_HOST_COPY_AUTO) mode = GG_HOST_COPY_STAGED;
    if (bytes < ((size_t)4 << 20) || mode == GG_HOST_COPY_DRIVER || host_pinned(src))
    {
        GG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
        return GG_OK;
    }
    if (mode == GG_HOST_COPY_DEVICE && host_page_tables() && (((uintptr_t)src | (uintptr_t)dst) & 15) == 0)
    {
        const size_t n16 = bytes / 16, tail = bytes - n16 * 16;
        k_copy_from_host<<<gg_sm_count() * 2, 1024, 0, s>>>((const uint4 *)src, (uint4 *)dst, n16);
        GG_CUDA(cudaGetLastError());
        if (tail)
            GG_CUDA(cudaMemcpyAsync((unsigned char *)dst + n16 * 16, (const unsigned char *)src + n16 * 16, tail,
                                    cudaMemcpyHostToDevice, s));
        return GG_OK;
    }
    std::lock_guard<std::mutex> lock(g_stage_mu);
    for (int b = 0; b < 2; b++)
        if (!g_stage[b])
        {
            GG_CUDA(cudaHostAlloc(&g_stage[b], STAGE_BYTES, cudaHostAllocDefault));
            GG_CUDA(cudaEventCreateWithFlags(&g_stage_ev[b], cudaEventDisableTiming));
        }
    bool used[2] = {false, false};
    for (size_t off = 0, i = 0; off < bytes; off += STAGE_BYTES, i++)
    {
        const int b = (int)(i & 1);
        if (used[b]) GG_CHECK(wait_event(g_stage_ev[b])); /* its last DMA has read the buffer */
        const size_t n = bytes - off < STAGE_BYTES ? bytes - off : STAGE_BYTES;
        parallel_copy(g_stage[b], (const unsigned char *)src + off, n);
        GG_CUDA(cudaMemcpyAsync((unsigned char *)dst + off, g_stage[b], n, cudaMemcpyHostToDevice, s));
        GG_CUDA(cudaEventRecord(g_stage_ev[b], s));
        used[b] = true;
    }
    /* the buffers go back to other callers only once their DMAs are done */
    for (int b = 0; b < 2; b++)
        if (used[b]) GG_CHECK(wait_event(g_stage_ev[b]));
    return GG_OK;
}

/* the pages at both ends of [p, p + n) are resident (a recycled array:
 * then the whole range is taken to be, and nothing needs touching) */
static bool ends_resident(const void *p, size_t n)
{
    static const size_t pg = [] {
        const long v = sysconf(_SC_PAGESIZE);
        return v > 0 ? (size_t)v : (size_t)4096;
    }();
    for (const uintptr_t a : {(uintptr_t)p, (uintptr_t)p + n - 1})
    {
        unsigned char in = 0;
        if (mincore((void *)(a / pg * pg), pg, &in) != 0 || !(in & 1)) return false;
    }
    return true;
}

void gg_host_dst_prepare(void *dst, size_t bytes)
{
    if (dst && bytes >= ((size_t)4 << 20) && host_page_tables() && !host_pinned(dst) && !ends_resident(dst, bytes))
        touch_pages(dst, bytes);
}

gg_status gg_copy_d2h(void *dst, const void *src, size_t bytes, cudaStream_t s)
{
    /* a copy to pageable memory blocks the host until the stream's earlier
     * work is done: wait for that work with the bounded poll first */
    const bool pinned = host_pinned(dst);
    if (!pinned)
    {
        gg_host_dst_prepare(dst, bytes);
        GG_CHECK(gg_wait(s));
    }
    if (bytes < ((size_t)4 << 20) || pinned || host_page_tables())
    {
        GG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s));
        return gg_wait(s);
    }
    std::lock_guard<std::mutex> lock(g_stage_mu);
    for (int b = 0; b < 2; b++)
        if (!g_stage[b])
        {
            GG_CUDA(cudaHostAlloc(&g_stage[b], STAGE_BYTES, cudaHostAllocDefault));
            GG_CUDA(cudaEventCreateWithFlags(&g_stage_ev[b], cudaEventDisableTiming));
        }
    /* chunk i lands in buffer i & 1; while it is in flight the previous
     * chunk is copied out by all host threads */
    const size_t nchunks = (bytes + STAGE_BYTES - 1) / STAGE_BYTES;
    for (size_t i = 0; i <= nchunks; i++)
    {
        if (i < nchunks)
        {
            const int b = (int)(i & 1);
            const size_t off = i * STAGE_BYTES, n = bytes - off < STAGE_BYTES ? bytes - off : STAGE_BYTES;
            GG_CUDA(cudaMemcpyAsync(g_stage[b], (const unsigned char *)src + off, n, cudaMemcpyDeviceToHost, s));
            GG_CUDA(cudaEventRecord(g_stage_ev[b], s));
        }
        if (i > 0)
        {
            const size_t k = i - 1;
            const int b = (int)(k & 1);
            const size_t off = k * STAGE_BYTES, n = bytes - off < STAGE_BYTES ? bytes - off : STAGE_BYTES;
            GG_CHECK(wait_event(g_stage_ev[b]));
            parallel_copy((unsigned char *)dst + off, g_stage[b], n);
        }
    }
    return GG_OK;
}

gg_status gg_event_at(gg_graph *g, uint32_t i, cudaEvent_t *out)
{
    if (i >= g->ev_count)
    {
        uint32_t n = g->ev_count ? g->ev_count : 64;
        while (n <= i) n *= 2;
        cudaEvent_t *p = (cudaEvent_t *)realloc(g->ev_pool, n * sizeof(cudaEvent_t));
        if (!p) return gg_fail(GG_ERR_NOMEM, "event pool");
        for (uint32_t k = g->ev_count; k < n; k++) GG_CUDA(cudaEventCreate(&p[k]));
        g->ev_pool = p;
        g->ev_count = n;
    }
    *out = g->ev_pool[i];
    return GG_OK;
}

float gg_event_ms(cudaEvent_t a, cudaEvent_t b)
{
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) return 0.0f;
    return ms;
}

/* ---- mapping ---------------------------------------------------------------- */

static gg_status upload(gg_graph *g, void **dst, const void *src, size_t bytes, size_t alloc_bytes,
                        cudaStream_t s)
{
    GG_CHECK(gg_dev_alloc(g, dst, alloc_bytes));
    if (bytes) GG_CHECK(gg_copy_h2d(*dst, src, bytes, s));
    if (alloc_bytes > bytes)
        GG_CUDA(cudaMemsetAsync((char *)*dst + bytes, 0, alloc_bytes - bytes, s));
    return GG_OK;
}


static gg_status map_arrays(gg_graph *g, const struct GraphCSR *graph, uint32_t what, cudaStream_t s)
{
    const uint32_t V = g->V, E = g->E;
    const size_t off_bytes = ((size_t)V + 1) * 4;
    const size_t edge_bytes = (size_t)E * 4, edge_alloc = ((size_t)E + GG_EDGE_PAD) * 4;
    if ((what & (GG_MAP_OUT | GG_MAP_IN)) && !g->out_deg)
    {
        if (!graph->vertices || !graph->vertices->out_degree)
            return gg_fail(GG_ERR_INVALID, "graph has no out_degree array");
        GG_CHECK(upload(g, (void **)&g->out_deg, graph->vertices->out_degree, (size_t)V * 4, (size_t)V * 4 + 16, s));
    }
    if ((what & GG_MAP_OUT) && !g->out_off)
    {
        if (!graph->vertices->edges_idx || !graph->sorted_edges_array || (E && !graph->sorted_edges_array->edges_array_dest))
            return gg_fail(GG_ERR_INVALID, "graph has no out-CSR arrays");
        /* offsets: edges_idx[0..V-1] plus the total E */
        GG_CHECK(upload(g, (void **)&g->out_off, graph->vertices->edges_idx, (size_t)V * 4, off_bytes, s));
        GG_CUDA(cudaMemcpyAsync(g->out_off + V, &g->E, 4, cudaMemcpyHostToDevice, s));
        GG_CHECK(upload(g, (void **)&g->out_adj, graph->sorted_edges_array->edges_array_dest, edge_bytes, edge_alloc, s));
    }
    if ((what & GG_MAP_IN) && !g->in_off)
    {
        if (!graph->inverse_vertices || !graph->inverse_vertices->edges_idx || !graph->inverse_sorted_edges_array ||
            (E && !graph->inverse_sorted_edges_array->edges_array_dest))
            return gg_fail(GG_ERR_INVALID, "graph has no inverse (CSC) arrays");
        GG_CHECK(upload(g, (void **)&g->in_off, graph->inverse_vertices->edges_idx, (size_t)V * 4, off_bytes, s));
        GG_CUDA(cudaMemcpyAsync(g->in_off + V, &g->E, 4, cudaMemcpyHostToDevice, s));
        GG_CHECK(upload(g, (void **)&g->in_adj, graph->inverse_sorted_edges_array->edges_array_dest, edge_bytes, edge_alloc, s));
    }
    if ((what & GG_MAP_OUT_W) && !g->out_w)
    {
        const float *w = graph->sorted_edges_array ? graph->sorted_edges_array->edges_array_weight : nullptr;
        if (w)
            GG_CHECK(upload(g, (void **)&g->out_w, w, edge_bytes, edge_alloc, s));
        else
            GG_CHECK(gg_fill_constant_weights(g, &g->out_w, E, s));
    }
    if ((what & GG_MAP_IN_W) && !g->in_w)
    {
        const float *w = graph->inverse_sorted_edges_array ? graph->inverse_sorted_edges_array->edges_array_weight : nullptr;
        if (w)
            GG_CHECK(upload(g, (void **)&g->in_w, w, edge_bytes, edge_alloc, s));
        else
            GG_CHECK(gg_fill_constant_weights(g, &g->in_w, E, s));
    }
    g->what |= what;
    /* the copies read pageable host memory; make them complete before the
     * caller may free or change it */
    return gg_wait(s);
}

__global__ void k_fill(float *p, size_t n, float v)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        p[i] = v;
}

gg_status gg_fill_constant_weights(gg_graph *g, float **dst, uint32_t E, cudaStream_t s)
{
    /* the reference's unweighted build multiplies by 0.0001f (SPMV.c:804) */
    GG_CHECK(gg_dev_alloc(g, (void **)dst, ((size_t)E + GG_EDGE_PAD) * 4));
    k_fill<<<gg_sm_count() * 4, 256, 0, s>>>(*dst, (size_t)E + GG_EDGE_PAD, 0.0001f);
    GG_CUDA(cudaGetLastError());
    return GG_OK;
}

gg_status gg_graph_new(uint32_t V, uint32_t E, gg_graph **out)
{
    *out = nullptr;
    int dev = 0;
    GG_CUDA(cudaGetDevice(&dev));
    gg_graph *g = new gg_graph();
    g->V = V;
    g->E = E;
    g->device = dev;
    cudaError_t e = cudaStreamCreateWithFlags(&g->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess)
    {
        delete g;
        return gg_cuda_fail(e, "cudaStreamCreate");
    }
    cudaEventCreate(&g->ev_begin);
    cudaEventCreate(&g->ev_end);
    *out = g;
    return GG_OK;
}

extern "C" gg_status gg_graph_map(const struct GraphCSR *graph, uint32_t what, void *stream, gg_graph **out)
{
    GgRange range("gg_graph_map");
    if (!out) return gg_fail(GG_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (!graph) return gg_fail(GG_ERR_INVALID, "graph is NULL");
    gg_graph *g = nullptr;
    GG_CHECK(gg_graph_new(graph->num_vertices, graph->num_edges, &g));
    g->max_weight = graph->max_weight;
    gg_status st = map_arrays(g, graph, what, gg_stream(g, stream));
    if (st != GG_OK)
    {
        std::string keep = t_last_error;
        gg_graph_unmap(g);
        t_last_error = keep;
        return st;
    }
    *out = g;
    return GG_OK;
}

static gg_status build_common(uint32_t V, uint32_t E, const uint32_t *src, const uint32_t *dst, const float *w,
                              bool host, float max_weight, uint32_t what, void *stream, gg_graph **out,
                              const uint32_t *label_host = nullptr)
{
    if (!out) return gg_fail(GG_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (V == 0) return gg_fail(GG_ERR_INVALID, "a graph needs at least one vertex");
    if (E && (!src || !dst)) return gg_fail(GG_ERR_INVALID, "edge arrays are NULL");
    if (!(what & (GG_MAP_OUT | GG_MAP_IN | GG_MAP_OUT_W | GG_MAP_IN_W)))
        return gg_fail(GG_ERR_INVALID, "nothing to build");
    gg_graph *g = nullptr;
    GG_CHECK(gg_graph_new(V, E, &g));
    cudaStream_t s = gg_stream(g, stream);
    uint32_t *ds = nullptr, *dd = nullptr;
    float *dw = nullptr;
    gg_status st = GG_OK;
    const bool want_w = w && (what & (GG_MAP_OUT_W | GG_MAP_IN_W));
    if (host)
    {
        /* the edge list to the device, freed once the build is done */
        st = upload(g, (void **)&ds, src, (size_t)E * 4, (size_t)E * 4 + 16, s);
        if (st == GG_OK) st = upload(g, (void **)&dd, dst, (size_t)E * 4, (size_t)E * 4 + 16, s);
        if (st == GG_OK && want_w) st = upload(g, (void **)&dw, w, (size_t)E * 4, (size_t)E * 4 + 16, s);
    }
    uint32_t *dl = nullptr;
    if (st == GG_OK && label_host)
    {
        /* relabel the uploaded ids in place: src' = label[src], dst' = label[dst] */
        st = upload(g, (void **)&dl, label_host, (size_t)V * 4, (size_t)V * 4 + 16, s);
        if (st == GG_OK) st = gg_check_permutation(g, dl, V, s);
        if (st == GG_OK && E) st = gg_apply_labels(ds, E, dl, ds, s);
        if (st == GG_OK && E) st = gg_apply_labels(dd, E, dl, dd, s);
    }
    if (st == GG_OK)
        st = gg_build_arrays(g, host ? ds : src, host ? dd : dst, want_w ? (host ? dw : w) : nullptr, what, s);
    if (dl)
    {
        gg_wait(s);
        gg_dev_free(g, dl, (size_t)V * 4 + 16);
    }
    if (host)
    {
        gg_wait(s);
        gg_dev_free(g, ds, (size_t)E * 4 + 16);
        gg_dev_free(g, dd, (size_t)E * 4 + 16);
        gg_dev_free(g, dw, (size_t)E * 4 + 16);
        if (st == GG_OK) g->max_weight = max_weight;
    }
    if (st != GG_OK)
    {
        std::string keep = t_last_error;
        gg_graph_unmap(g);
        t_last_error = keep;
        return st;
    }
    *out = g;
    return GG_OK;
}

extern "C" gg_status gg_graph_build(const struct EdgeList *edges, uint32_t what, void *stream, gg_graph **out)
{
    if (!edges) return gg_fail(GG_ERR_INVALID, "edge list is NULL");
    return build_common(edges->num_vertices, edges->num_edges, edges->edges_array_src, edges->edges_array_dest,
                        edges->edges_array_weight, true, edges->max_weight, what, stream, out);
}

extern "C" gg_status gg_graph_build_relabelled(const struct EdgeList *edges, const uint32_t *label_array,
                                               uint32_t what, void *stream, gg_graph **out)
{
    if (!edges || !label_array) return gg_fail(GG_ERR_INVALID, "NULL argument");
    return build_common(edges->num_vertices, edges->num_edges, edges->edges_array_src, edges->edges_array_dest,
                        edges->edges_array_weight, true, edges->max_weight, what, stream, out, label_array);
}

extern "C" gg_status gg_relabel_order(const struct EdgeList *edges, uint32_t lmode, uint64_t seed,
                                      uint32_t *label_array, void *stream)
{
    if (!edges || !label_array) return gg_fail(GG_ERR_INVALID, "NULL argument");
    const uint32_t V = edges->num_vertices, E = edges->num_edges;
    if (V == 0) return GG_OK;
    if (E && (!edges->edges_array_src || !edges->edges_array_dest)) return gg_fail(GG_ERR_INVALID, "edge arrays are NULL");
    gg_graph *g = nullptr;
    GG_CHECK(gg_graph_new(V, E, &g));
    cudaStream_t s = gg_stream(g, stream);
    uint32_t *ds = nullptr, *dd = nullptr, *dl = nullptr;
    gg_status st = upload(g, (void **)&ds, edges->edges_array_src, (size_t)E * 4, (size_t)E * 4 + 16, s);
    if (st == GG_OK) st = upload(g, (void **)&dd, edges->edges_array_dest, (size_t)E * 4, (size_t)E * 4 + 16, s);
    if (st == GG_OK) st = gg_dev_alloc(g, (void **)&dl, (size_t)V * 4 + 16);
    if (st == GG_OK) st = gg_relabel_device(g, V, E, ds, dd, lmode, seed, dl, s);
    if (st == GG_OK) st = gg_wait(s);
    if (st == GG_OK && cudaMemcpyAsync(label_array, dl, (size_t)V * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        st = gg_fail(GG_ERR_CUDA, "cudaMemcpyAsync");
    if (st == GG_OK) st = gg_wait(s);
    gg_wait(s);
    gg_dev_free(g, ds, (size_t)E * 4 + 16);
    gg_dev_free(g, dd, (size_t)E * 4 + 16);
    gg_dev_free(g, dl, (size_t)V * 4 + 16);
    std::string keep = t_last_error;
    gg_graph_unmap(g);
    t_last_error = keep;
    return st;
}

extern "C" gg_status gg_graph_build_device(uint32_t num_vertices, uint32_t num_edges, const uint32_t *src,
                                           const uint32_t *dst, const float *weights, uint32_t what, void *stream,
                                           gg_graph **out)
{
    return build_common(num_vertices, num_edges, src, dst, weights, false, 0.0f, what, stream, out);
}

extern "C" gg_status gg_graph_download(const gg_graph *gc, uint32_t *out_idx, uint32_t *out_adj, float *out_w,
                                       uint32_t *in_idx, uint32_t *in_adj, float *in_w, float *max_weight)
{
    if (!gc) return gg_fail(GG_ERR_INVALID, "graph is NULL");
    gg_graph *g = const_cast<gg_graph *>(gc);
    cudaStream_t s = g->own_stream;
    const size_t vb = (size_t)g->V * 4, eb = (size_t)g->E * 4;
    struct Part
    {
        void *host;
        const void *dev;
        size_t bytes;
        const char *what;
    } parts[] = {{out_idx, g->out_off, vb, "out-CSR"}, {out_adj, g->out_adj, eb, "out-CSR"},
                 {out_w, g->out_w, eb, "out-edge weights"}, {in_idx, g->in_off, vb, "CSC"},
                 {in_adj, g->in_adj, eb, "CSC"}, {in_w, g->in_w, eb, "in-edge weights"}};
    GG_CHECK(gg_wait(s)); /* bounded, before copies to pageable memory */
    for (const Part &p : parts)
    {
        if (!p.host) continue;
        if (!p.dev) return gg_fail(GG_ERR_INVALID, std::string("the mapping has no ") + p.what);
        if (p.bytes) GG_CUDA(cudaMemcpyAsync(p.host, p.dev, p.bytes, cudaMemcpyDeviceToHost, s));
    }
    if (max_weight) *max_weight = g->max_weight;
    return gg_wait(s);
}

extern "C" gg_status gg_graph_share(const gg_graph *src, gg_graph **out)
{
    if (!out) return gg_fail(GG_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (!src) return gg_fail(GG_ERR_INVALID, "src is NULL");
    gg_graph *g = new gg_graph();
    g->V = src->V;
    g->E = src->E;
    g->what = src->what;
    g->max_weight = src->max_weight;
    g->device = src->device;
    g->owns_arrays = false;
    g->out_off = src->out_off; g->out_adj = src->out_adj; g->out_w = src->out_w;
    g->in_off = src->in_off; g->in_adj = src->in_adj; g->in_w = src->in_w;
    g->out_deg = src->out_deg;
    /* the launch shapes tuned for the graph */
    g->pr_shape = src->pr_shape;
    g->spmv_shape = src->spmv_shape;
    g->bfs_heavy = src->bfs_heavy;
    g->ppr_tile = src->ppr_tile;
    g->graphs_cfg = src->graphs_cfg;
    g->tuned = src->tuned;
    g->tune_looked_up = src->tune_looked_up;
    cudaError_t e = cudaStreamCreateWithFlags(&g->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess)
    {
        delete g;
        return gg_cuda_fail(e, "cudaStreamCreate");
    }
    cudaEventCreate(&g->ev_begin);
    cudaEventCreate(&g->ev_end);
    *out = g;
    return GG_OK;
}

extern "C" gg_status gg_graph_extend(gg_graph *g, const struct GraphCSR *graph, uint32_t what, void *stream)
{
    if (!g || !graph) return gg_fail(GG_ERR_INVALID, "NULL argument");
    if (!g->owns_arrays) return gg_fail(GG_ERR_INVALID, "a shared view cannot be extended");
    if (graph->num_vertices != g->V || graph->num_edges != g->E)
        return gg_fail(GG_ERR_INVALID, "graph size differs from the mapping");
    return map_arrays(g, graph, what, gg_stream(g, stream));
}

static void free_tiles(gg_graph *g, gg_tiles &t, bool idle)
{
    dev_release(g, t.coord, ((size_t)t.ntiles + 1) * sizeof(uint2), idle);
    t = gg_tiles();
}

extern "C" gg_status gg_graph_unmap(gg_graph *g)
{
    if (!g) return GG_OK;
    /* the mapping's device is current while its blocks are released (the
     * caller's current device is restored at the end) */
    int caller_dev = -1;
    if (cudaGetDevice(&caller_dev) != cudaSuccess) cudaGetLastError();
    if (caller_dev != g->device) cudaSetDevice(g->device);
    if (g->own_stream) cudaStreamSynchronize(g->own_stream);
    /* once for all the blocks below (work of calls on callers' streams
     * included); if it fails, each block is freed on its own */
    const bool idle = cudaDeviceSynchronize() == cudaSuccess;
    if (!idle) cudaGetLastError();
    const size_t off_bytes = ((size_t)g->V + 1) * 4, edge_alloc = ((size_t)g->E + GG_EDGE_PAD) * 4;
    if (g->owns_arrays)
    {
        dev_release(g, g->out_off, off_bytes, idle);
        dev_release(g, g->out_adj, edge_alloc, idle);
        dev_release(g, g->out_w, edge_alloc, idle);
        dev_release(g, g->in_off, off_bytes, idle);
        dev_release(g, g->in_adj, edge_alloc, idle);
        dev_release(g, g->in_w, edge_alloc, idle);
        dev_release(g, g->out_deg, (size_t)g->V * 4 + 16, idle);
    }
    for (int i = 0; i < 3; i++)
    {
        dev_release(g, g->in_w16[i], edge_alloc, idle);
        dev_release(g, g->out_w16[i], edge_alloc, idle);
    }
    free_tiles(g, g->in_tiles, idle);
    free_tiles(g, g->out_tiles, idle);
    free_tiles(g, g->ppr_tiles, idle);
    dev_release(g, g->hot_adj, ((size_t)g->E + GG_EDGE_PAD) * 4, idle);
    dev_release(g, g->hot_list, (size_t)GG_HOT_ENTRIES * 4, idle);
    free_tiles(g, g->hot_tiles, idle);
    for (auto &b : g->work) dev_release(g, b.ptr, b.bytes, idle);
    dev_release(g, g->graphs.coord, g->graphs.bytes, idle);
    if (g->pinned) cudaFreeHost(g->pinned);
    if (g->pr_exec) cudaGraphExecDestroy(g->pr_exec);
    for (uint32_t i = 0; i < g->ev_count; i++) cudaEventDestroy(g->ev_pool[i]);
    free(g->ev_pool);
    if (g->ev_begin) cudaEventDestroy(g->ev_begin);
    if (g->ev_end) cudaEventDestroy(g->ev_end);
    if (g->own_stream) cudaStreamDestroy(g->own_stream);
    const int dev = g->device;
    delete g;
    if (caller_dev >= 0 && caller_dev != dev) cudaSetDevice(caller_dev);
    return GG_OK;
}

extern "C" size_t gg_graph_device_bytes(const gg_graph *g) { return g ? g->device_bytes : 0; }

gg_status gg_tiles_get(gg_graph *g, int in, cudaStream_t s, gg_tiles **out)
{
    gg_tiles &t = in ? g->in_tiles : g->out_tiles;
    const uint32_t *off = in ? g->in_off : g->out_off;
    if (!off) return gg_fail(GG_ERR_INVALID, in ? "mapping has no CSC arrays" : "mapping has no CSR arrays");
    if (!t.coord)
    {
        const uint64_t items = (uint64_t)g->V + g->E;
        const uint64_t nt = (items + GG_TILE_ITEMS - 1) / GG_TILE_ITEMS;
        if (nt >= 0xffffffffull) return gg_fail(GG_ERR_INVALID, "graph too large for 32-bit tile ids");
        t.ntiles = (uint32_t)(nt ? nt : 1);
        GG_CHECK(gg_dev_alloc(g, (void **)&t.coord, ((size_t)t.ntiles + 1) * sizeof(uint2)));
        GG_CHECK(gg_launch_tile_coords(off, g->V, g->E, t.ntiles, t.coord, s));
    }
    *out = &t;
    return GG_OK;
}

gg_status gg_weights16(gg_graph *g, int in, int storage, cudaStream_t s, const void **out)
{
    if (storage != GG_STORE_BF16 && storage != GG_STORE_F16)
        return gg_fail(GG_ERR_INVALID, "not a 16-bit storage");
    void *&slot = in ? g->in_w16[storage] : g->out_w16[storage];
    const float *w = in ? g->in_w : g->out_w;
    if (!w) return gg_fail(GG_ERR_INVALID, "mapping has no edge weights");
    if (!slot)
    {
        GG_CHECK(gg_dev_alloc(g, &slot, ((size_t)g->E + GG_EDGE_PAD) * 4));
        GG_CHECK(gg_launch_to_half(w, slot, (size_t)g->E + GG_EDGE_PAD, storage, s));
    }
    *out = slot;
    return GG_OK;
}

/* ---- small kernels used by the runtime ------------------------------------------- */

__global__ void k_tile_coords(const uint32_t *__restrict__ off, uint32_t V, uint32_t E, uint32_t ntiles,
                              uint32_t tile_items, uint2 *__restrict__ coord)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t > ntiles) return;
    const uint64_t items = (uint64_t)V + E;
    uint64_t d = (uint64_t)t * tile_items;
    if (d > items) d = items;
    /* rows ended before diagonal d: largest i with off[i] + (i-1) < d over row ends off[1..V] */
    uint64_t lo = d > E ? d - E : 0, hi = d < V ? d : V;
    while (lo < hi)
    {
        uint64_t mid = (lo + hi) >> 1;
        if ((uint64_t)off[mid + 1] + mid < d)
            lo = mid + 1;
        else
            hi = mid;
    }
    coord[t] = make_uint2((uint32_t)lo, (uint32_t)(d - lo));
}

gg_status gg_launch_tile_coords(const uint32_t *off, uint32_t V, uint32_t E, uint32_t ntiles, uint2 *coord,
                                cudaStream_t s, uint32_t tile_items)
{
    const uint32_t n = ntiles + 1;
    k_tile_coords<<<(n + 255) / 256, 256, 0, s>>>(off, V, E, ntiles, tile_items, coord);
    GG_CUDA(cudaGetLastError());
    return GG_OK;
}

__global__ void k_to_half(const float *__restrict__ src, void *__restrict__ dst, size_t n, int storage)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    {
        if (storage == GG_STORE_BF16)
            ((__nv_bfloat16 *)dst)[i] = __float2bfloat16_rn(src[i]);
        else
            ((__half *)dst)[i] = __float2half_rn(src[i]);
    }
}

gg_status gg_launch_to_half(const float *src, void *dst, size_t n, int storage, cudaStream_t s)
{
    k_to_half<<<gg_sm_count() * 4, 256, 0, s>>>(src, dst, n, storage);
    GG_CUDA(cudaGetLastError());
    return GG_OK;
}
