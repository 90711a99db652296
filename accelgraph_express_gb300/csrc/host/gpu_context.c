/*
 * Device context of the drop-in entry points: side options, the resident
 * mapping cache keyed by GraphCSR pointer, error reporting and host-memory
 * pinning.  The reference has no handle to hang device copies on (its
 * functions take a bare GraphCSR*, pageRank.h:69-86), so resident copies are
 * keyed by the pointer and dropped with graphGpuRelease.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>
#include <time.h>

#include <cuda_runtime_api.h>

#include "gg_host.h"

static pthread_mutex_t g_lock = PTHREAD_MUTEX_INITIALIZER;
static GraphGpuOptions g_opts = {GG_STORE_F32, 0, 0, 0};
static __thread gg_status t_last = GG_OK;
static int g_device_ready = -1; /* -1 unknown, 0 no device, 1 ready */

#define MAX_RESIDENT 64
static struct { struct GraphCSR *graph; gg_graph *g; } g_resident[MAX_RESIDENT];

#define MAX_PINNED 256
static void *g_pinned[MAX_PINNED];

#define HOST_CACHE_SLOTS 8
#define HOST_CACHE_MIN ((size_t)64 << 10)
#define HOST_CACHE_MAX ((size_t)1 << 30)
static pthread_mutex_t g_host_cache_lock = PTHREAD_MUTEX_INITIALIZER;
static struct { void *p; size_t bytes; } g_host_cache[HOST_CACHE_SLOTS];
static size_t g_host_cache_bytes = 0;

void *gg_host_array_take(size_t bytes)
{
    if (bytes >= HOST_CACHE_MIN)
    {
        pthread_mutex_lock(&g_host_cache_lock);
        for (int i = 0; i < HOST_CACHE_SLOTS; i++)
            if (g_host_cache[i].p && g_host_cache[i].bytes == bytes)
            {
                void *p = g_host_cache[i].p;
                g_host_cache[i].p = NULL;
                g_host_cache_bytes -= bytes;
                pthread_mutex_unlock(&g_host_cache_lock);
                return p;
            }
        pthread_mutex_unlock(&g_host_cache_lock);
    }
    return malloc(bytes);
}

void gg_host_array_give(void *p, size_t bytes)
{
    if (!p) return;
    if (bytes >= HOST_CACHE_MIN && bytes <= HOST_CACHE_MAX)
    {
        pthread_mutex_lock(&g_host_cache_lock);
        if (g_host_cache_bytes + bytes <= HOST_CACHE_MAX)
            for (int i = 0; i < HOST_CACHE_SLOTS; i++)
                if (!g_host_cache[i].p)
                {
                    g_host_cache[i].p = p;
                    g_host_cache[i].bytes = bytes;
                    g_host_cache_bytes += bytes;
                    pthread_mutex_unlock(&g_host_cache_lock);
                    return;
                }
        pthread_mutex_unlock(&g_host_cache_lock);
    }
    free(p);
}

double gg_seconds(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + (double)ts.tv_nsec * 1e-9;
}

void graphGpuSetOptions(const GraphGpuOptions *opts)
{
    if (!opts) return;
    pthread_mutex_lock(&g_lock);
    g_opts = *opts;
    g_device_ready = -1;
    pthread_mutex_unlock(&g_lock);
}

void graphGpuGetOptions(GraphGpuOptions *opts)
{
    if (opts) *opts = g_opts;
}

const GraphGpuOptions *gpu_options(void) { return &g_opts; }

gg_status graphGpuLastError(void) { return t_last; }

void gpu_report(const char *where, gg_status st)
{
    t_last = st;
    fprintf(stderr, "accelgraph-gb300: %s failed (status %d): %s\n", where, (int)st, gg_last_error());
}

static gg_status ensure_device(void)
{
    if (g_device_ready == 1) return GG_OK;
    gg_status st = gg_device_init(g_opts.device);
    g_device_ready = st == GG_OK ? 1 : 0;
    return st;
}

gg_graph *gpu_acquire(struct GraphCSR *graph, uint32_t what, int force_resident)
{
    t_last = GG_OK;
    pthread_mutex_lock(&g_lock);
    gg_status st = ensure_device();
    if (st != GG_OK)
    {
        pthread_mutex_unlock(&g_lock);
        gpu_report("device init", st);
        return NULL;
    }
    gg_graph *g = NULL;
    if (g_opts.keep_resident || force_resident)
    {
        int slot = -1, empty = -1;
        for (int i = 0; i < MAX_RESIDENT; i++)
        {
            if (g_resident[i].graph == graph) { slot = i; break; }
            if (!g_resident[i].graph && empty < 0) empty = i;
        }
        if (slot >= 0)
        {
            g = g_resident[slot].g;
            st = gg_graph_extend(g, graph, what, NULL);
        }
        else
        {
            st = gg_graph_map(graph, what, NULL, &g);
            if (st == GG_OK && empty >= 0)
            {
                g_resident[empty].graph = graph;
                g_resident[empty].g = g;
            }
        }
    }
    else
        st = gg_graph_map(graph, what, NULL, &g);
    pthread_mutex_unlock(&g_lock);
    if (st != GG_OK)
    {
        gpu_report("graph upload", st);
        return NULL;
    }
    return g;
}

void gpu_release_call(struct GraphCSR *graph, gg_graph *g)
{
    if (!g) return;
    pthread_mutex_lock(&g_lock);
    int resident = 0;
    for (int i = 0; i < MAX_RESIDENT; i++)
        if (g_resident[i].graph == graph && g_resident[i].g == g) resident = 1;
    pthread_mutex_unlock(&g_lock);
    if (!resident) gg_graph_unmap(g);
}

void graphGpuRelease(struct GraphCSR *graph)
{
    pthread_mutex_lock(&g_lock);
    for (int i = 0; i < MAX_RESIDENT; i++)
        if (g_resident[i].graph == graph)
        {
            gg_graph_unmap(g_resident[i].g);
            g_resident[i].graph = NULL;
            g_resident[i].g = NULL;
        }
    pthread_mutex_unlock(&g_lock);
}

void gg_host_pin(void *p, size_t bytes)
{
    if (!p || bytes < (1u << 20)) return;
    const char *env = getenv("GG_PIN_HOST");
    if (env && env[0] == '0') return;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0)
    {
        cudaGetLastError();
        return;
    }
    pthread_mutex_lock(&g_lock);
    int slot = -1;
    for (int i = 0; i < MAX_PINNED; i++)
        if (!g_pinned[i]) { slot = i; break; }
    if (slot >= 0 && cudaHostRegister(p, bytes, cudaHostRegisterDefault) == cudaSuccess)
        g_pinned[slot] = p;
    else
        cudaGetLastError();
    pthread_mutex_unlock(&g_lock);
}

void gg_host_unpin(void *p)
{
    if (!p) return;
    pthread_mutex_lock(&g_lock);
    for (int i = 0; i < MAX_PINNED; i++)
        if (g_pinned[i] == p)
        {
            cudaHostUnregister(p);
            g_pinned[i] = NULL;
        }
    pthread_mutex_unlock(&g_lock);
}
