#ifndef GG_SERVER_H
#define GG_SERVER_H

/*
 * gg_server: a query server over one device-resident graph (no counterpart
 * in the reference, whose entry points run one algorithm per call).  Clients
 * submit personalised-PageRank queries (a seed set) and BFS queries (a
 * source) from any thread; two worker threads drain them on the GPU:
 *
 *   PPR  continuous batching: one running batch of up to max_ppr_batch
 *        vector slots (64 at most) advances every busy slot by one iteration
 *        per round (one gather over the first 16, 32 or 64 slots, as the busy
 *        ones need); between rounds waiting queries are admitted into free
 *        slots and slots that ran all their iterations retire, so a query
 *        waits at most one round before it starts, and its latency is about
 *        its own iterations;
 *   BFS  bfs_workers workers (default 2), each running one direction-
 *        optimising gg_bfs per query on its own shared view of the graph
 *        and stream, so searches overlap each other and the PPR rounds.
 *
 * Results stay in device memory until the client takes them.  Admission is
 * by a device-memory budget: a worker starts work only while the results
 * held (taken or not) plus the new ones fit mem_budget_bytes (PPR: 4V bytes
 * per query, BFS: 8V), so a client that does not take results slows the
 * server down instead of exhausting the GPU.  A query's result does not
 * depend on the queries batched or running with it (a PPR vector is
 * bit-identical to gg_ppr's for that seed set alone, whatever slots run
 * beside it; BFS levels are exact).
 */

#include <stdint.h>
#include <stddef.h>

#include "gg_runtime.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gg_server gg_server;

typedef struct gg_server_params
{
    uint32_t max_ppr_batch;     /* vectors per PPR launch, 1..64 */
    uint32_t ppr_iterations;    /* >= 1 */
    float damp;                 /* 0.85 */
    uint32_t ppr_storage;       /* GG_STORE_F32 or GG_STORE_BF16 */
    uint64_t mem_budget_bytes;  /* device bytes for results held; at least 8V */
    uint32_t bfs_workers;       /* concurrent BFS workers, 0: 2 (at most 16) */
} gg_server_params;

enum { GG_QUERY_PPR = 0, GG_QUERY_BFS = 1 };

typedef struct gg_query_info
{
    uint32_t kind;              /* GG_QUERY_PPR / GG_QUERY_BFS */
    uint32_t status;            /* gg_status of the query's run */
    double submit_s;            /* host steady-clock seconds */
    double start_s;             /* its run was launched */
    double done_s;              /* its result was complete in device memory */
    uint32_t batch_size;        /* PPR: busy slots of the running batch when it was admitted */
    uint32_t bfs_levels;        /* BFS: frontier steps run */
    uint32_t bfs_reached;       /* BFS: vertices reached, source included */
} gg_query_info;

/* Start workers over `g` (a mapping with GG_MAP_IN and, for BFS, GG_MAP_OUT;
 * the server uses it and a view of it until gg_server_stop). */
gg_status gg_server_start(gg_graph *g, const gg_server_params *p, gg_server **out);
/* Queue a PPR query from `nseeds` seed vertices (copied; repeats weigh) or
 * a BFS query from `source`; *ticket identifies it. */
gg_status gg_server_submit_ppr(gg_server *s, const uint32_t *seeds, uint32_t nseeds, uint64_t *ticket);
gg_status gg_server_submit_bfs(gg_server *s, uint32_t source, uint64_t *ticket);
/* Wait up to timeout_ms for the query, copy its result into the host
 * buffers given (PPR: V floats of ranks; BFS: V parents and V distances, the
 * values gg_bfs returns) and release it.  GG_ETIMEDOUT leaves the query in
 * place; an unknown ticket is GG_ERR_INVALID. */
gg_status gg_server_take(gg_server *s, uint64_t ticket, uint32_t timeout_ms, gg_query_info *info, float *ppr,
                         int32_t *parents, uint32_t *distances);
/* Finish the queued queries, stop the workers, free every result. */
gg_status gg_server_stop(gg_server *s);

#ifdef __cplusplus
}
#endif

#endif
