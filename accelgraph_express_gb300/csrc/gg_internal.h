/*
 * Internal declarations shared by the gg_runtime translation units.
 * Not part of the public ABI (include/gg_runtime.h is).
 */
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <cstdint>
#include <cstddef>
#include <string>
#include <vector>

#include "gg_runtime.h"

/* Merge-path tiles are consumed by single warps: one warp takes a tile of
 * GG_TILE_ITEMS = 32 * GG_TILE_IPT merge items (row ends + edges), so no
 * CTA-wide barrier sits on the hot path.  IPT is odd so that the lanes'
 * reads of the staged values hit distinct shared-memory banks.  Kernels run
 * persistent CTAs of GG_TILE_WARPS warps that stride over the tiles; small
 * CTAs keep each one's static shared staging (double-buffered row offsets,
 * values and row sums for every warp) under 48 KB. */
#define GG_TILE_IPT 9
#define GG_TILE_ITEMS (32 * GG_TILE_IPT)
#define GG_TILE_WARPS 4
#define GG_TILE_NT (32 * GG_TILE_WARPS)

/* Slack after every edge array so 16-byte vector loads of the last group
 * stay inside the allocation. */
#define GG_EDGE_PAD 16

struct gg_tiles
{
    uint32_t ntiles = 0;
    uint2 *coord = nullptr;   /* ntiles+1 merge-path coordinates (row, edge) */
};

/* Growable device scratch owned by a mapping. */
struct gg_buf
{
    void *ptr = nullptr;
    size_t bytes = 0;
};

/* Launch shape of an FP pull gather (PageRank, SpMV): the default, set by
 * gg_autotune, or found in the tuning cache for a graph like this one. */
struct gg_pull_shape
{
    uint32_t hot = 2;        /* hot-vertex table: 0 off, 1 on, 2 by size (from 1M vertices) */
    uint32_t ctas = 5;       /* plain kernel: resident CTAs per SM (GG_PULL_CTAS_PER_SM) */
    uint32_t hot_warps = 32; /* hot kernel: warps of its one CTA per SM (GG_HOT_WARPS) */
};

/* Configuration of the many-graphs PageRank kernel (graphs.cu): tile items
 * per lane (5, 7 or 9), warps per CTA, and the bin threshold: graphs of at
 * most smem_vmax vertices keep contributions and sums in shared memory. */
struct gg_graphs_config
{
    uint32_t ipt = 7, warps = 16, smem_vmax = 4096;
    uint32_t ctas = 2; /* resident CTAs per SM: the shared-memory carve-out holds just these, the rest is L1 */
    /* without an epsilon stop: 0 the union pull (default), 1 the
     * many-graphs kernel, 2 the union pull (tuned); with one, always the
     * many-graphs kernel */
    uint32_t strategy = 0;
};

/* The many-graphs run's preparation, cached on the mapping for the graph
 * boundaries it was made for: per-graph tile coordinates and the size order
 * (one device allocation at coord: voff, cbase, order, then the tiles). */
struct gg_graphs_state
{
    uint32_t ngraphs = 0, items = 0;
    std::vector<uint32_t> h_voff;
    void *coord = nullptr;
    size_t bytes = 0;
    const uint32_t *voff = nullptr, *cbase = nullptr, *order = nullptr;
    uint2 *tiles = nullptr;
};

struct gg_graph
{
    uint32_t V = 0, E = 0;
    uint32_t what = 0;
    float max_weight = 0.0f; /* the edge list's, kept for host copies */
    /* false for a view made by gg_graph_share: the graph arrays belong to
     * the mapping it was made from */
    bool owns_arrays = true;
    int device = 0;
    cudaStream_t own_stream = nullptr;

    /* out-CSR */
    uint32_t *out_off = nullptr;
    uint32_t *out_adj = nullptr;
    float *out_w = nullptr;
    /* in-CSR (CSC) */
    uint32_t *in_off = nullptr;
    uint32_t *in_adj = nullptr;
    float *in_w = nullptr;
    uint32_t *out_deg = nullptr;

    gg_tiles in_tiles;   /* tiles over the CSC (pull) */
    gg_tiles out_tiles;  /* tiles over the CSR (push) */

    /* bf16/f16 copies of the edge weights, made on first use */
    void *in_w16[3] = {nullptr, nullptr, nullptr};
    void *out_w16[3] = {nullptr, nullptr, nullptr};

    /* work buffers, grown on demand */
    gg_buf work[32];
    /* merge-path tiles of the batched PageRank gather (own tile size) */
    gg_tiles ppr_tiles;
    const float *ppr_ranks = nullptr;
    uint32_t ppr_stride = 0;
    /* hot-vertex table: flag-encoded copy of in_adj and the slot -> vertex list */
    uint32_t *hot_adj = nullptr;
    uint32_t *hot_list = nullptr;  /* GG_HOT_ENTRIES slots */
    uint32_t hot_n = 0;            /* slots in use */
    uint32_t hot_cap = 0;          /* table capacity the encoding was made for */
    gg_tiles hot_tiles;            /* tiles of 32 * GG_HOT_IPT items over the CSC */
    /* page-locked host scratch for small per-step read-backs */
    void *pinned = nullptr;
    size_t pinned_bytes = 0;

    /* bumped whenever device memory of the mapping is freed (a work buffer
     * regrown, scratch released): a cached CUDA graph recorded at another
     * generation may point at freed memory and is captured again */
    uint64_t mem_gen = 0;
    /* the last GG_PR_CUDA_GRAPH call, instantiated, with the parameters it
     * was captured for */
    cudaGraphExec_t pr_exec = nullptr;
    unsigned char pr_key[64] = {};
    uint64_t pr_gen = 0;
    uint32_t pr_launches = 0, pr_gather_launches = 0;

    cudaEvent_t ev_begin = nullptr, ev_end = nullptr;
    /* timing events reused across calls (profile mode) */
    cudaEvent_t *ev_pool = nullptr;
    uint32_t ev_count = 0;
    size_t device_bytes = 0;
    const float *last_ranks = nullptr;
    /* the last many-graphs run: preparation and per-graph iteration counts */
    gg_graphs_state graphs;
    const uint32_t *graphs_iters = nullptr;
    uint32_t graphs_n = 0;
    /* the many-graphs configuration in force (default, set, or tuned) */
    gg_graphs_config graphs_cfg;
    /* tuned launch shapes (tune.cu): the pull gathers, the BFS heavy-vertex
     * threshold, the batched PPR tile; tuned = bit per family */
    gg_pull_shape pr_shape, spmv_shape;
    uint32_t bfs_heavy = 64;
    uint32_t ppr_tile = 512, ppr_tiles_items = 0;
    uint32_t tuned = 0;
    bool tune_looked_up = false;
};

/* error state */
gg_status gg_fail(gg_status s, const std::string &msg);
gg_status gg_cuda_fail(cudaError_t e, const char *what);
#define GG_CUDA(call)                                                   \
    do {                                                                \
        cudaError_t e_ = (call);                                        \
        if (e_ != cudaSuccess) return gg_cuda_fail(e_, #call);          \
    } while (0)
#define GG_CHECK(expr)                                                  \
    do {                                                                \
        gg_status s_ = (expr);                                          \
        if (s_ != GG_OK) return s_;                                     \
    } while (0)

/* a kernel launch that may begin while the previous kernel on the stream
 * still runs (programmatic dependent launch): the kernel must call
 * pdl_wait() (gg_device.cuh) before it touches that kernel's output */
template <typename... KArgs, typename... Args>
inline cudaError_t gg_launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                                 Args &&...args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

/* device memory helpers (account into g->device_bytes) */
gg_status gg_dev_alloc(gg_graph *g, void **p, size_t bytes);
void gg_dev_free(gg_graph *g, void *p, size_t bytes);
/* work buffer slot `slot`, at least `bytes` long (contents undefined) */
gg_status gg_work(gg_graph *g, int slot, size_t bytes, void **out);
/* a mapping with its stream and events and no arrays */
gg_status gg_graph_new(uint32_t V, uint32_t E, gg_graph **out);
/* E + GG_EDGE_PAD weights of the reference's constant 0.0001f */
gg_status gg_fill_constant_weights(gg_graph *g, float **dst, uint32_t E, cudaStream_t s);
/* CSR/CSC of `g` from device edge arrays (build.cu) */
gg_status gg_build_arrays(gg_graph *g, const uint32_t *src, const uint32_t *dst, const float *w, uint32_t what,
                          cudaStream_t s);
/* relabelling (build.cu): label[orig] = new for the reference's -l modes
 * 0..10 over device edge ids; a permutation check; ids -> labels */
gg_status gg_relabel_device(gg_graph *g, uint32_t V, uint64_t E, const uint32_t *src, const uint32_t *dst,
                            uint32_t mode, uint64_t seed, uint32_t *label, cudaStream_t s);
gg_status gg_check_permutation(gg_graph *g, const uint32_t *label, uint32_t V, cudaStream_t s);
gg_status gg_apply_labels(const uint32_t *ids, uint64_t n, const uint32_t *label, uint32_t *out, cudaStream_t s);
/* the mapping's page-locked host scratch, at least `bytes` long */
gg_status gg_pinned(gg_graph *g, size_t bytes, void **out);
/* build the hot-vertex table of the mapping for a table of `cap` entries
 * (<= GG_HOT_ENTRIES; rebuilt only when cap changes; needs GG_MAP_IN), and
 * the tiles of the hot kernels */
gg_status gg_hot_prepare(gg_graph *g, cudaStream_t s, uint32_t cap);
cudaStream_t gg_stream(gg_graph *g, void *user_stream);
/* host wait on all work queued on `s`, bounded by the wait limit */
gg_status gg_wait(cudaStream_t s);

/* an NVTX range for the lifetime of a scope: each entry point is one named
 * range in Nsight timelines (a no-op while no tool is attached) */
struct GgRange
{
    explicit GgRange(const char *name) { nvtxRangePushA(name); }
    ~GgRange() { nvtxRangePop(); }
    GgRange(const GgRange &) = delete;
    GgRange &operator=(const GgRange &) = delete;
};
/* host -> device copy (returns with the copy queued on s; the source must
 * stay valid until s reaches it); pageable sources are read by a kernel
 * where the device uses the host page tables, else go through page-locked
 * staging filled by all host threads */
gg_status gg_copy_h2d(void *dst, const void *src, size_t bytes, cudaStream_t s);
/* device -> host copy, complete on return (waits for s); pageable
 * destinations are written by the driver's copy where the device uses the
 * host page tables, else filled from page-locked staging by all host
 * threads */
gg_status gg_copy_d2h(void *dst, const void *src, size_t bytes, cudaStream_t s);
/* make a pageable destination of a coming device -> host copy resident (one
 * store per page on all host threads; its contents become undefined), so
 * the copy runs at the DMA rate; called while the device still computes the
 * data, it overlaps that work.  A no-op for page-locked memory, below 4 MB,
 * and where the device does not use the host page tables. */
void gg_host_dst_prepare(void *dst, size_t bytes);
/* tiles of the CSC (in = 1) or CSR (in = 0), computed on first use */
gg_status gg_tiles_get(gg_graph *g, int in, cudaStream_t s, gg_tiles **out);
/* bf16 (storage 1) / f16 (storage 2) copy of the in- or out-edge weights */
gg_status gg_weights16(gg_graph *g, int in, int storage, cudaStream_t s, const void **out);
/* the i-th pooled timing event of g, created on first use */
gg_status gg_event_at(gg_graph *g, uint32_t i, cudaEvent_t *out);
/* elapsed ms between two events recorded on s (after a wait) */
float gg_event_ms(cudaEvent_t a, cudaEvent_t b);

/* launch helpers implemented in the kernel translation units */
/* coord[t] = (rows ended, edges consumed) at merge diagonal t * tile_items */
gg_status gg_launch_tile_coords(const uint32_t *off, uint32_t V, uint32_t E, uint32_t ntiles,
                                uint2 *coord, cudaStream_t s, uint32_t tile_items = GG_TILE_ITEMS);
gg_status gg_launch_to_half(const float *src, void *dst, size_t n, int storage, cudaStream_t s);
int gg_sm_count();
/* persistent grid for a tile kernel: one CTA per resident slot, no more
 * CTAs than tiles need.  ctas_per_sm > 0 caps the resident CTAs per SM and
 * sets the kernel's shared-memory carve-out to just hold them, so the rest
 * of each SM's combined L1/shared array caches the gathered values. */
int gg_persistent_grid(const void *kernel, uint32_t ntiles, int ctas_per_sm = 0);
/* resident blocks per SM of `kernel` at this block size and dynamic shared
 * memory (cudaOccupancyMaxActiveBlocksPerMultiprocessor, remembered; 0 on
 * failure); for kernels whose attributes do not change between launches */
int gg_occupancy(const void *kernel, int threads, size_t smem);

/* Resident CTAs per SM of the pull gathers.  Measured on GB300 for R-MAT
 * scale 22-24 PageRank and SpMV pulls: fewer CTAs leave more L1 for the hot
 * in-neighbours' values (skewed graphs concentrate most gathers on a few
 * thousand sectors); more hide more latency. */
#define GG_PULL_CTAS_PER_SM 5

/* control block bytes of gg::grid_barrier (gg_device.cuh) */
#define GG_BAR_BYTES (4096 + 128 * 16)
/* device-side wait limit of the grid barriers, in ns (gg_set_barrier_limit_us) */
unsigned long long gg_barrier_limit_ns();

/* Hot-vertex table of the pull gather (hot.cu): up to GG_HOT_ENTRIES
 * vertices with the most out-edges are read from a shared-memory table of
 * GG_HOT_TABLE_BYTES (as many entries as the stored value type fits: 8K FP32,
 * 16K BF16/FP16); a copy of the CSC ids marks them as GG_HOT_FLAG | slot.
 * The kernels that use it run one CTA of GG_HOT_WARPS warps per SM sharing
 * the table (measured on R-MAT-24: many warps per SM matter more than a
 * bigger table or longer tiles). */
#define GG_HOT_FLAG 0x80000000u
#define GG_HOT_ENTRIES 16384u
#define GG_HOT_TABLE_BYTES 32768u
#define GG_HOT_WARPS 32
#define GG_HOT_IPT 7
/* many-graphs PageRank (graphs.cu): tile coordinates and size order for the
 * graph boundaries h_voff (cached on the mapping), and the one launch */
gg_status gg_graphs_prepare(gg_graph *g, uint32_t ngraphs, const uint32_t *h_voff, uint32_t items, cudaStream_t s);
gg_status gg_graphs_launch(gg_graph *g, const gg_graphs_config &cfg, uint32_t ngraphs, const gg_pr_params *p,
                           float eps_f, float *rank, uint32_t *counter, uint32_t *iters, uint32_t *active, double *err,
                           cudaStream_t s);
size_t gg_graphs_tile_items(const gg_graphs_config &cfg);
/* the configuration a many-graphs run on g uses */
gg_graphs_config gg_graphs_choice(gg_graph *g, uint32_t ngraphs);
/* tuning (tune.cu): apply the process's tuning cache to g once (the shapes
 * tuned earlier for a graph of the same size class on this GPU) */
void gg_tune_lookup(gg_graph *g, cudaStream_t s);

/* One iteration of the batched personalised PageRank on caller-held state
 * (ppr.cu; the server's continuous batch): the first kp (16/32/64) vectors
 * of rows of rs values; vectors in rank_mask write their ranks, vectors in
 * zero_mask store zero contributions (their slot is freed). */
struct gg_ppr_round_args
{
    uint32_t kp = 16; /* rows hold 64 values */
    int bf16 = 0;
    const void *cin = nullptr;
    void *cout = nullptr;
    float *rank = nullptr;
    unsigned long long rank_mask = 0, zero_mask = 0;
    const uint32_t *seed_idx = nullptr;
    const float *tele = nullptr;
    float *slots = nullptr;
    float damp = 0.85f;
};
/* tiles and the two contribution buffers (zeroed) and the tile slots */
gg_status gg_ppr_round_prepare(gg_graph *g, uint32_t rs, int bf16, void **cb0, void **cb1, float **slots,
                               cudaStream_t s);
/* seed indices of the seed vertices, and iteration-0 contributions of the
 * vectors in `fresh` at them (their columns must be zero elsewhere) */
gg_status gg_ppr_round_seed(gg_graph *g, uint32_t rs, int bf16, void *cin, const uint32_t *d_seedv, uint32_t nseedv,
                            const float *d_init, uint32_t *d_seed_idx, unsigned long long fresh, cudaStream_t s);
gg_status gg_ppr_round(gg_graph *g, const gg_ppr_round_args &r, cudaStream_t s);

/* smallest float f with (double)f >= x, and largest float f with (double)f <= x */
float gg_float_ceil(double x);
float gg_float_floor(double x);
