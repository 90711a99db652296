#ifndef GG_RUNTIME_H
#define GG_RUNTIME_H

/*
 * gg_runtime: the thin C ABI between the CSR algorithm entry points and the
 * GB300 kernels.  It replaces the reference's CAPI offload layer
 * (02_capi_graph/include/capi_utils/capienv.h:146-166,
 *  02_capi_graph/src/capi_utils/capienv.c):
 *
 *   reference (capienv.c)                      here
 *   -----------------------------------------  -----------------------------
 *   mapGraphCSRToWED      :396-438             gg_graph_map
 *   setupAFUGraphCSR      :30-55               gg_device_init (+ gg_graph_map)
 *   startAFU / startCU    :58-109              gg_pagerank / gg_bfs / gg_spmv
 *   waitAFU (unbounded)   :111-172             bounded wait inside each call,
 *                                              GG_ETIMEDOUT after the limit
 *   readCmdResponseStats  :174-201             per-call result structs
 *                                              (kernel time, launches)
 *   releaseAFU            :299-303             gg_graph_unmap
 *
 * All entry points are plain C: host pointers, sizes, an opaque graph handle
 * and an optional CUDA stream passed as `void *` (NULL = the library's own
 * stream).  Every call returns a gg_status; gg_last_error() gives a message.
 * Calls on one gg_graph must not overlap; different graphs may be used from
 * different host threads.
 */

#include <stdint.h>
#include <stddef.h>

#include "graphCSR.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gg_status
{
    GG_OK = 0,
    GG_ERR_INVALID = 1,    /* bad argument (size, source, mode, missing array) */
    GG_ERR_NO_DEVICE = 2,  /* no CUDA device / driver */
    GG_ERR_CUDA = 3,       /* CUDA runtime error */
    GG_ERR_NOMEM = 4,      /* device or host allocation failed */
    GG_ETIMEDOUT = 5,      /* device work did not finish within the wait limit */
    GG_ERR_KERNEL = 6      /* a kernel reported an error through its status word */
} gg_status;

typedef struct gg_graph gg_graph;

/* Arrays a mapping must carry (bit mask). */
#define GG_MAP_OUT    0x1u   /* out-CSR: edges_idx, out_degree, edges_array_dest */
#define GG_MAP_IN     0x2u   /* in-CSR (CSC): inverse edges_idx, in-degree, in-neighbours; out_degree */
#define GG_MAP_OUT_W  0x4u   /* out-edge weights (constant 0.0001f when the graph has none) */
#define GG_MAP_IN_W   0x8u   /* in-edge weights */
#define GG_MAP_ALL    0xFu

/* Storage type of the gathered vertex values (PageRank contributions, SpMV
 * x) and of SpMV edge weights.  Accumulation is always FP32. */
typedef enum gg_storage
{
    GG_STORE_F32 = 0,
    GG_STORE_BF16 = 1,
    GG_STORE_F16 = 2
} gg_storage;

/* ---- device and graph ----------------------------------------------------- */

gg_status gg_device_init(int device);
const char *gg_last_error(void);
/* Upper bound, in milliseconds, of every host wait on device work
 * (default 120000, env GG_WAIT_TIMEOUT_MS). */
void gg_set_wait_timeout_ms(uint32_t ms);
/* Upper bound, in microseconds, of each device-side wait of the grid
 * barriers inside the single-launch kernels (direction-optimising BFS,
 * batched personalised PageRank); default 2,000,000 (2 s), 0 restores it.
 * A wait that runs out ends the launch early and the call returns
 * GG_ERR_KERNEL with the context intact.  For diagnostics and tests of
 * that path: at a few microseconds the barriers give up before the other
 * blocks arrive. */
void gg_set_barrier_limit_us(uint32_t us);
/* How copies from pageable host memory (4 MB and more) reach HBM:
 *   GG_HOST_COPY_AUTO    the default: GG_HOST_COPY_STAGED (the direct routes
 *                        are faster once a buffer has been copied, but the
 *                        first direct copy of a buffer was several times
 *                        slower on a Grace host);
 *   GG_HOST_COPY_STAGED  32 MB chunks through two page-locked buffers, each
 *                        filled by all host threads while the other's DMA runs;
 *   GG_HOST_COPY_DRIVER  one cudaMemcpyAsync from the pageable memory;
 *   GG_HOST_COPY_DEVICE  a kernel reads the pageable memory in place (only
 *                        where the device uses the host's page tables and
 *                        source and destination are 16-byte aligned, else
 *                        staged).
 * Env GG_HOST_COPY (auto / staged / driver / device) sets the initial mode.
 * Copies to pageable memory use the driver's copy where the device uses the
 * host's page tables, else staging. */
#define GG_HOST_COPY_AUTO 0u
#define GG_HOST_COPY_STAGED 1u
#define GG_HOST_COPY_DRIVER 2u
#define GG_HOST_COPY_DEVICE 3u
void gg_set_host_copy_mode(uint32_t mode);
uint32_t gg_host_copy_mode(void);

/* Copy the arrays selected by `what` to HBM.  Offsets are padded so that
 * every array starts on a 256-byte boundary.  The host graph is only read. */
gg_status gg_graph_map(const struct GraphCSR *graph, uint32_t what, void *stream, gg_graph **out);
/* A second handle on the same device graph (no copy): its own stream and
 * work buffers, so calls on `src` and on the view may run concurrently.
 * The view must be unmapped before `src`; it cannot be extended. */
gg_status gg_graph_share(const gg_graph *src, gg_graph **out);
/* Upload any arrays in `what` that the mapping does not carry yet. */
gg_status gg_graph_extend(gg_graph *g, const struct GraphCSR *graph, uint32_t what, void *stream);
gg_status gg_graph_unmap(gg_graph *g);

/* Build the CSR and CSC on the device from an edge list, in place of the
 * host sort + assignment (the reference's OpenGraph sortRunAlgorithms +
 * graphCSRAssignEdgeList, called at SSSP.c:552-565 and bellmanFord.c:737-744;
 * their sources are absent from the snapshot).  A stable LSD radix sort of
 * (row << b | neighbour) words, b = bits for V, as graphCSRFromEdgeList does
 * on the host: every array equals that build's.  `what` as for gg_graph_map;
 * out-degrees always come along.  _W without weights gives the constant
 * 0.0001f.  An id >= num_vertices is GG_ERR_INVALID.
 * gg_graph_build reads a host EdgeList; gg_graph_build_device takes device
 * arrays of num_edges entries (`weights` may be NULL) and records the largest
 * weight above 0 as max_weight. */
gg_status gg_graph_build(const struct EdgeList *edges, uint32_t what, void *stream, gg_graph **out);
gg_status gg_graph_build_device(uint32_t num_vertices, uint32_t num_edges, const uint32_t *src, const uint32_t *dst,
                                const float *weights, uint32_t what, void *stream, gg_graph **out);
/* Degree-based relabelling (the reference's -l modes, README.md:362-378,
 * code in the absent OpenGraph submodule), computed on the GPU from the edge
 * list: label_array[orig] = new id (V entries, host).  lmode: 0 identity,
 * 1 out-degree, 2 in-degree, 3 (in+out)-degree (descending degree), 4/5 DBG
 * out/in (degree-based grouping: eight groups, group k >= 1 the degrees in
 * [avg/2 * 2^(k-1), avg/2 * 2^k), hotter groups first), 6/7 HUBSort out/in
 * (hubs, degree > E/V, by descending degree, then the rest), 8/9 HUBCluster
 * out/in (hubs, then the rest), 10 random (SplitMix64(seed ^ id)).  Ties and
 * groups keep the original order.  Mode 11 (labels from a file) needs no
 * computation: pass those labels to gg_graph_build_relabelled. */
gg_status gg_relabel_order(const struct EdgeList *edges, uint32_t lmode, uint64_t seed, uint32_t *label_array,
                           void *stream);
/* gg_graph_build of the edge list with every id replaced by
 * label_array[id] (which must be a permutation of 0..V-1). */
gg_status gg_graph_build_relabelled(const struct EdgeList *edges, const uint32_t *label_array, uint32_t what,
                                    void *stream, gg_graph **out);
/* Copy a mapping's arrays to host buffers (any may be NULL): row offsets
 * (V entries, as edges_idx), neighbours and weights (E entries) of the
 * out-CSR and the CSC, and the edge list's max_weight. */
gg_status gg_graph_download(const gg_graph *g, uint32_t *out_idx, uint32_t *out_adj, float *out_w, uint32_t *in_idx,
                            uint32_t *in_adj, float *in_w, float *max_weight);
/* Bytes of device memory held by the mapping (graph + work buffers). */
size_t gg_graph_device_bytes(const gg_graph *g);
/* Device memory the library has freed is kept for reuse (a mapping made
 * and dropped per call then pays no cudaMalloc / cudaFree), up to
 * GG_DEVICE_CACHE_MB (default 16384) MB; an allocation that fails empties
 * the cache first.  trim hands every cached block back to CUDA; bytes is
 * what the cache holds now. */
void gg_device_cache_trim(void);
size_t gg_device_cache_bytes(void);

/* ---- PageRank --------------------------------------------------------------- */

/* Modes use the reference's pushpull codes (pageRank.c:879-935). */
typedef enum gg_pr_mode
{
    GG_PR_PULL = 0, GG_PR_PUSH = 1, GG_PR_PULL_FX64 = 2, GG_PR_PUSH_FX64 = 3,
    GG_PR_PULL_Q32 = 4, GG_PR_PUSH_Q = 5, GG_PR_DD_PULL = 6, GG_PR_DD_PUSH = 7,
    GG_PR_DD_PULLPUSH = 8, GG_PR_PULL_FX32 = 9, GG_PR_PULL_FX16 = 10,
    GG_PR_PULL_FX8 = 11, GG_PR_PULL_Q16 = 12, GG_PR_PULL_Q8 = 13
} gg_pr_mode;

typedef struct gg_pr_params
{
    uint32_t mode;            /* gg_pr_mode */
    uint32_t storage;         /* gg_storage of the gathered contributions (pull/push FP modes) */
    uint32_t max_iterations;
    uint32_t init_one_over_n; /* 0: reference (start 0.15, divide by V at the end); 1: start 1/V, rank = 0.15/V + 0.85*sum, no final division */
    double epsilon;
    float damp;               /* 0.85f in the reference */
    uint32_t profile;         /* 1: time every gather launch with CUDA events */
    uint32_t flags;           /* GG_PR_CUDA_GRAPH, GG_PR_HOT_OFF, GG_PR_HOT_ON, GG_PR_BATCH_UNION */
} gg_pr_params;

/* Run the whole call (initialisation, every iteration, normalisation) as
 * one CUDA graph launch; per-launch timing (profile) is not available then.
 * The instantiated graph stays with the mapping: a later call with the same
 * parameters relaunches it, unless device memory of the mapping has been
 * freed since (another algorithm regrowing a shared work buffer), in which
 * case it is captured again. */
#define GG_PR_CUDA_GRAPH 0x1u
/* The pull gather of the FP32/BF16/FP16 modes serves the contributions of
 * the 16K vertices with the most out-edges from a shared-memory table (built
 * once per mapping; an extra copy of the CSC ids).  By default from 1M
 * vertices up; HOT_OFF never, HOT_ON on any graph.  Results are the same. */
#define GG_PR_HOT_OFF 0x2u
#define GG_PR_HOT_ON 0x4u
/* gg_pagerank_batch: run the ordinary pull over the union of the graphs
 * (every graph iterates until all have converged) instead of the
 * many-graphs kernel (FP32 pull: one CTA per graph, each graph with its own
 * stop, every iteration in one launch). */
#define GG_PR_BATCH_UNION 0x8u

typedef struct gg_pr_result
{
    uint32_t iterations;      /* reference convention (see pageRank.h) */
    uint32_t active;          /* active vertices in the last iteration run */
    double error_total;       /* last iteration's sum |delta| / V */
    double rank_sum;          /* sum of the returned ranks */
    float gather_ms;          /* profile: summed device time of the gather launches */
    uint32_t gather_launches; /* gather launches timed */
    uint32_t launches;        /* kernels launched by the call */
    uint32_t hot_table;       /* 1: the gather read the hot-vertex table (GG_PR_HOT_*) */
} gg_pr_result;

/* Run PageRank on a mapping that carries GG_MAP_IN (pull) or GG_MAP_OUT (push).
 * `ranks` (host, V floats) receives the final ranks when not NULL. */
gg_status gg_pagerank(gg_graph *g, const gg_pr_params *p, float *ranks, gg_pr_result *r, void *stream);
/* Device pointer to the last run's final ranks (V floats), valid until the
 * next call on `g`. */
const float *gg_pagerank_device_ranks(const gg_graph *g);
/* PageRank over a mapping that is the union of `ngraphs` graphs occupying
 * vertex ranges vertex_off[i] .. vertex_off[i+1] (host array, ngraphs+1
 * entries, from 0 to V; no counterpart in the reference), every graph
 * ranked as if alone (each vertex divided by its own graph's vertex count).
 * The reference formulation only (init_one_over_n = 0).
 * FP32 pull with an epsilon stop, or with the many-graphs strategy
 * (gg_pagerank_batch_strategy, gg_autotune): the many-graphs kernel, one
 * launch for every graph and every iteration; one CTA per graph (largest
 * first), small graphs' contributions in shared memory
 * (gg_pagerank_batch_config / gg_autotune pick the bin threshold and tile
 * shape); every graph stops on its own (iteration counts from
 * gg_pagerank_batch_iterations); the result carries the largest count, the
 * largest error_total and the active vertices of graphs that ran out.  The
 * edges must stay inside their graph's range (GG_ERR_INVALID otherwise).
 * Otherwise (other modes, GG_PR_BATCH_UNION, FP32 without an epsilon stop
 * by default): the iterations of gg_pagerank over the union, the stop rule
 * and error_total over the union. */
gg_status gg_pagerank_batch(gg_graph *g, const gg_pr_params *p, uint32_t ngraphs, const uint32_t *vertex_off,
                            float *ranks, gg_pr_result *r, void *stream);
/* Per-graph iteration counts (the reference's convention) of the last
 * many-graphs run of gg_pagerank_batch on g, which had `ngraphs` graphs. */
gg_status gg_pagerank_batch_iterations(const gg_graph *g, uint32_t ngraphs, uint32_t *iterations);
/* Shape of the many-graphs kernel on g: merge items per lane of its tiles
 * (5, 7 or 9), warps per CTA (1..32), the bin threshold (graphs of at most
 * smem_vmax vertices keep contributions and sums in shared memory; 0: none)
 * and the resident CTAs per SM (the shared-memory carve-out holds just
 * these; the rest of the SM's array is L1).  Default 7, 16, 4096, 2;
 * gg_autotune picks one per mapping. */
gg_status gg_pagerank_batch_config(gg_graph *g, uint32_t ipt, uint32_t warps, uint32_t smem_vmax,
                                   uint32_t ctas_per_sm);
/* Which FP32 pull gg_pagerank_batch runs on g when epsilon is 0 (every
 * graph runs all iterations either way): 0 the union pull (the default;
 * measured faster on R-MAT mixes), 1 the many-graphs kernel, 2 the union
 * pull.  With an epsilon stop the many-graphs kernel always runs, so that
 * every graph stops on its own. */
gg_status gg_pagerank_batch_strategy(gg_graph *g, uint32_t strategy);

/* ---- BFS -------------------------------------------------------------------- */

typedef enum gg_bfs_mode
{
    GG_BFS_PULL = 0, GG_BFS_PUSH = 1, GG_BFS_DO = 2, GG_BFS_PUSH_BITMAP = 3, GG_BFS_DO_BITMAP = 4
} gg_bfs_mode;

typedef struct gg_bfs_params
{
    uint32_t mode;            /* gg_bfs_mode */
    uint32_t source;          /* internal vertex id (already relabelled) */
    uint32_t alpha;           /* 15 in the reference (BFS.c:564) */
    uint32_t beta;            /* 18 in the reference (BFS.c:565) */
    uint32_t profile;
} gg_bfs_params;

typedef struct gg_bfs_result
{
    uint32_t processed_nodes; /* vertices reached, the source included (BFS.c:368 counts it) */
    uint32_t levels;          /* frontier steps run */
    uint32_t top_down_steps;
    uint32_t bottom_up_steps;
    uint64_t edges_examined;  /* adjacency entries read by all steps */
    float step_ms;            /* profile: summed device time of the step kernels */
    uint32_t launches;
} gg_bfs_result;

/* Needs GG_MAP_OUT for top-down steps and GG_MAP_IN for bottom-up steps.
 * `parents` (int32, V) and `distances` (uint32, V) are host outputs (may be NULL). */
gg_status gg_bfs(gg_graph *g, const gg_bfs_params *p, int32_t *parents, uint32_t *distances,
                 gg_bfs_result *r, void *stream);

/* Device pointers to the last gg_bfs's parents and distances on `g` (V
 * entries each, the same values gg_bfs copies out), valid until the next
 * call on `g`. */
gg_status gg_bfs_device_results(const gg_graph *g, const int32_t **parents, const uint32_t **distances);

/* ---- connected components ------------------------------------------------- */

/* Algorithms use the reference's pushpull codes for connected components
 * (connectedComponents.c:337-360). */
typedef enum gg_cc_algorithm
{
    GG_CC_SHILOACH_VISHKIN = 0, GG_CC_AFFOREST = 1, GG_CC_WEAKLY = 2
} gg_cc_algorithm;

typedef struct gg_cc_params
{
    uint32_t algorithm;       /* gg_cc_algorithm */
    uint32_t neighbor_rounds; /* Afforest sampling rounds; 0 = 2 (the reference's) */
    uint32_t samples;         /* Afforest labels sampled to find the largest component; 0 = 1024 */
    uint32_t use_in_edges;    /* Afforest final link over the CSC too: 0 no (the caller declares the graph
                                 symmetric), 1 yes (needs GG_MAP_IN), 2 when mapped (else nothing is skipped) */
    uint32_t max_iterations;  /* Shiloach-Vishkin / weakly: give up after this many (0 = V + 1) */
    uint32_t profile;         /* 1: time the kernels with CUDA events */
    uint64_t seed;            /* Afforest sample (SplitMix64) */
} gg_cc_params;

typedef struct gg_cc_result
{
    uint32_t iterations;      /* hook / propagation rounds run (Afforest: neighbor_rounds) */
    uint32_t components;      /* distinct labels */
    uint32_t launches;
    uint32_t skipped_label;   /* Afforest: the sampled component left out of the final link, or ~0 */
    float kernel_ms;          /* profile */
} gg_cc_result;

/* Label every vertex with the smallest vertex id of its weakly connected
 * component (edges taken without direction); `components` (V entries, host,
 * may be NULL).  Needs GG_MAP_OUT; Afforest uses the CSC as `use_in_edges`
 * says. */
gg_status gg_cc(gg_graph *g, const gg_cc_params *p, uint32_t *components, gg_cc_result *r, void *stream);
/* Device pointer to the last gg_cc's labels on `g` (V entries), valid until
 * the next call on `g`. */
gg_status gg_cc_device_labels(const gg_graph *g, const uint32_t **components);

/* One frontier step on host state, for the reference's step functions.
 * direction 0: top-down from `frontier` (a queue of `frontier_len` ids when
 * `frontier_is_bitmap` is 0, else a bitmap of ceil(V/32) words);
 * direction 1: bottom-up from the bitmap `frontier`.
 * parents/distances are read and updated in place; the next frontier is
 * written as a queue (`next_queue`, may be NULL) and/or a bitmap
 * (`next_bitmap`, may be NULL); *next_len receives its size and *counter
 * receives mf (top-down) or nf (bottom-up). */
gg_status gg_bfs_step_host(gg_graph *g, int direction, const uint32_t *frontier, uint32_t frontier_len,
                           int frontier_is_bitmap, int32_t *parents, uint32_t *distances,
                           uint32_t *next_queue, uint32_t *next_bitmap, uint32_t *next_len,
                           uint32_t *counter, void *stream);

/* ---- SpMV ------------------------------------------------------------------- */

typedef enum gg_spmv_mode
{
    GG_SPMV_PULL = 0, GG_SPMV_PUSH = 1, GG_SPMV_PULL_FX = 2, GG_SPMV_PUSH_FX = 3
} gg_spmv_mode;

typedef struct gg_spmv_params
{
    uint32_t mode;            /* gg_spmv_mode */
    uint32_t storage;         /* gg_storage of x and of the edge weights (pull/push FP modes) */
    uint32_t iterations;
    uint32_t profile;
    uint32_t flags;           /* GG_PR_HOT_OFF / GG_PR_HOT_ON: the hot-vertex table for the FP pull */
} gg_spmv_params;

typedef struct gg_spmv_result
{
    double checksum;          /* sum of round2(y[v]) as the reference prints (SPMV.c:727-730) */
    float spmv_ms;            /* profile: summed device time of the product launches */
    uint32_t spmv_launches;
    uint32_t launches;
} gg_spmv_result;

/* Pull needs GG_MAP_IN|GG_MAP_IN_W, push GG_MAP_OUT|GG_MAP_OUT_W.
 * `x` (host, V) is the input vector, or NULL for the reference's
 * x[v] = 1/outdeg(v) (0.001 when 0); `x_out` receives the x used; `y`
 * receives the result.  Any of them may be NULL. */
gg_status gg_spmv(gg_graph *g, const gg_spmv_params *p, const float *x, float *x_out, float *y,
                  gg_spmv_result *r, void *stream);

/*
 * Allocation-free SpMV pull, y = A^T x, for callers that must not allocate
 * GPU memory (no counterpart in the reference): a plugin whose host owns
 * every device allocation, a real-time loop where cudaMalloc could block,
 * or a process whose device memory is reserved up front.  All arrays are the
 * caller's DEVICE pointers: in_off (V+1 offsets of the inverse CSR, with
 * in_off[V] = E), in_src (E in-neighbours), w (E FP32 weights), x (V), y (V,
 * overwritten).  in_off must be non-decreasing with in_off[V] = E: the
 * kernels trust it, and other offsets are undefined behaviour (reads past
 * in_src and w).  y must not overlap x, w, in_off or in_src (GG_ERR_INVALID
 * when it does).  The call allocates nothing: its scratch is a 4 MiB array
 * inside the library that every GPU loading the library holds until the
 * process exits, so V + E must not exceed gg_spmv_pull_noalloc_max_items()
 * (GG_ERR_INVALID otherwise).  Every call looks up the array's device
 * address in the context current at the call (a context that was reset or
 * replaced gets the new address); the first call in a context also loads
 * the library's kernels into it, so make that first call before any stream
 * capture.  Calls share the one array: calls whose work overlaps on the GPU
 * (other streams, other host threads) race and must be serialised by the
 * caller.  Work is queued on `stream` (NULL: the legacy default stream) and
 * not waited for.
 */
gg_status gg_spmv_pull_noalloc(uint32_t V, uint32_t E, const uint32_t *in_off, const uint32_t *in_src,
                               const float *w, const float *x, float *y, void *stream);
/* Largest V + E that gg_spmv_pull_noalloc accepts. */
uint64_t gg_spmv_pull_noalloc_max_items(void);

/* ---- batched personalised PageRank -------------------------------------------- */

/*
 * K personalised PageRank vectors over one graph, advanced together by one
 * pull gather per iteration (no counterpart in the reference's C API; per
 * vector it is the pull PageRank of pageRank.c:1026-1069 with the teleport
 * going to the vector's seed set S_k instead of every vertex):
 *     rank_0(v)  = c(v)/|S_k|,   rank'(v) = (1-d) c(v)/|S_k| + d * sum_{u->v} rank(u)/outdeg(u)
 * where c(v) counts v in S_k (seeds may repeat).  Exactly `iterations`
 * iterations run (no convergence test).  Needs GG_MAP_IN.
 */
typedef struct gg_ppr_params
{
    uint32_t num_vectors;     /* K, 1..64 */
    uint32_t iterations;      /* >= 1 */
    float damp;               /* 0.85 */
    uint32_t storage;         /* GG_STORE_F32 or GG_STORE_BF16 contributions; sums are FP32 */
    uint32_t profile;         /* 1: time every gather launch */
} gg_ppr_params;

typedef struct gg_ppr_result
{
    float gather_ms;          /* profile: summed device time of the gather launches */
    uint32_t gather_launches;
    uint32_t launches;
    uint32_t padded_vectors;  /* vectors per vertex row on the device: 16, 32 or 64 */
    uint32_t persistent;      /* 1: every iteration ran in one cooperative launch (profile off) */
} gg_ppr_result;

/* Seeds of vector k are seeds[seed_off[k] .. seed_off[k+1]) (host arrays,
 * K+1 offsets, seed_off[0] = 0).  `ranks` (host, V*K floats, vertex-major:
 * ranks[v*K + k]) receives the result when not NULL. */
gg_status gg_ppr(gg_graph *g, const gg_ppr_params *p, const uint32_t *seed_off, const uint32_t *seeds,
                 float *ranks, gg_ppr_result *r, void *stream);
/* Device pointer to the last gg_ppr's ranks (V rows of *stride floats),
 * valid until the next call on `g`. */
const float *gg_ppr_device_ranks(const gg_graph *g, uint32_t *stride);

/* ---- autotuner ----------------------------------------------------------------
 * No counterpart in the reference (its one run-time granularity knob is
 * binSize, graphConfig.h:18).  gg_autotune times candidate launch shapes of
 * the hot kernels on a mapping and keeps the fastest on it (the default
 * shape is always a candidate); the picks are also remembered per graph
 * class (size, mean degree, degree skew, SM count), so the first call on a
 * later mapping of a graph of the same class starts with them, and
 * gg_tune_save / gg_tune_load carry them to another process.
 *   GG_TUNE_PR, GG_TUNE_SPMV  FP pull gather: hot-vertex table off with 3-8
 *                             CTAs per SM, or on with 16/24/32 warps
 *   GG_TUNE_BFS               top-down heavy-vertex threshold (32..1024)
 *   GG_TUNE_PPR               batched personalised PageRank tile (256/512/1024)
 *   GG_TUNE_BATCH             many graphs: the union pull or the many-graphs
 *                             kernel, and the kernel's shape (CTAs per SM and
 *                             warps, shared-memory bin threshold, items per
 *                             lane; needs vertex_off)
 */
#define GG_TUNE_PR 0x1u
#define GG_TUNE_SPMV 0x2u
#define GG_TUNE_BFS 0x4u
#define GG_TUNE_PPR 0x8u
#define GG_TUNE_BATCH 0x10u

typedef struct gg_tune_params
{
    uint32_t families;          /* GG_TUNE_* bits */
    uint32_t storage;           /* gg_storage the PR / SpMV / PPR candidates run with */
    uint32_t reps;              /* timed runs per candidate after one untimed run (0: 3) */
    uint32_t ngraphs;           /* GG_TUNE_BATCH: graphs of the batch */
    const uint32_t *vertex_off; /* GG_TUNE_BATCH: their vertex ranges (host, ngraphs + 1) */
} gg_tune_params;

typedef struct gg_tune_choice
{
    uint32_t family;      /* GG_TUNE_* */
    uint32_t params[5];   /* PR/SPMV: hot (0/1), CTAs per SM, hot warps; BFS: threshold; PPR: tile;
                             BATCH: items per lane, warps, bin threshold, CTAs per SM, strategy
                             (1 the many-graphs kernel, 2 the union pull) */
    float default_ms;     /* median time of the default shape */
    float tuned_ms;       /* median time of the pick */
    uint32_t candidates;  /* shapes timed */
} gg_tune_choice;

typedef struct gg_tune_result
{
    gg_tune_choice choice[5];
    uint32_t n;
} gg_tune_result;

gg_status gg_autotune(gg_graph *g, const gg_tune_params *p, gg_tune_result *r, void *stream);
/* The remembered picks of this process, as text lines; load adds them. */
gg_status gg_tune_save(const char *path);
gg_status gg_tune_load(const char *path);
/* Forget the remembered picks (mappings keep the shapes they have). */
gg_status gg_tune_reset(void);
/* The shape g uses now for one family (params as in gg_tune_choice; a
 * mapping that has not run the family yet may still pick up a remembered
 * shape on its first call). */
gg_status gg_tune_get(const gg_graph *g, uint32_t family, uint32_t *params);

/* ---- drop-in side options ---------------------------------------------------- */

/*
 * GPU-only knobs for the reference-compatible entry points, kept out of
 * `struct Arguments` so its layout stays the reference's.  Defaults:
 * storage FP32, device 0, graph re-uploaded on every call.
 */
typedef struct GraphGpuOptions
{
    uint32_t storage;         /* gg_storage for PageRank/SpMV gathers */
    int device;
    uint32_t keep_resident;   /* 1: keep each GraphCSR's device copy between calls (graphGpuRelease frees it) */
    uint32_t verbose;         /* 1: print the reference's iteration tables */
} GraphGpuOptions;

void graphGpuSetOptions(const GraphGpuOptions *opts);
void graphGpuGetOptions(GraphGpuOptions *opts);
/* Status of the last failed drop-in call (GG_OK if none). */
gg_status graphGpuLastError(void);
/* Drop the resident device copy of `graph`, if any. */
void graphGpuRelease(struct GraphCSR *graph);

#ifdef __cplusplus
}
#endif

#endif
