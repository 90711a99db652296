#ifndef ORACLE_H
#define ORACLE_H

/*
 * CPU oracle for the CSR traversal hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's algorithms
 * (02_capi_graph/src/algorithms/capi/{pageRank,BFS,SPMV}.c) used to check
 * the GPU path, to generate golden fixtures and as the timed CPU baseline.
 * Nothing in the product library links or calls it.  Every function cites
 * the reference lines it follows.  It has its own R-MAT generator and CSR
 * builder so that the product's builder is checked independently.
 *
 * Pinning: the restatement is checked against the reference's own C code,
 * compiled from the reference sources with stand-in headers for its missing
 * OpenGraph submodule (oracle/build_ref.sh -> oracle/_ref/), on the
 * reference's fixture graphs and on small R-MAT graphs; the outputs are
 * committed under tests/golden/.  The FPGA-offloaded loops (PageRank and SpMV
 * pull) exist in the reference only as SystemVerilog, so for those the
 * gather is restated from the RTL (cu_sum_kernel_control.sv) and only the
 * host passes around it are pinned.  The fixed-point and quantisation
 * formats live in the missing OpenGraph headers; the formats defined by
 * the orc_fx* and orc_quant* functions below are this project's and those variants are unpinned.
 *
 * All functions are sequential and deterministic when nthreads <= 1; with
 * nthreads > 1 they use OpenMP the way the reference does (schedule
 * (dynamic,1024) vertex loops, CAS claims in top-down BFS, atomic scatters in
 * push), for the CPU baseline timing.
 */

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_csr
{
    uint32_t V;
    uint32_t E;
    const uint32_t *out_off;  /* V+1, CSR by source */
    const uint32_t *out_adj;  /* E destinations */
    const float *out_w;       /* E or NULL */
    const uint32_t *in_off;   /* V+1, CSC by destination */
    const uint32_t *in_adj;   /* E sources */
    const float *in_w;        /* E or NULL */
} orc_csr;

/* ---- graph construction ------------------------------------------------- */

uint64_t orc_splitmix64(uint64_t x);
/* R-MAT edges [first, first+count) of the generator described in graphCSR.h */
void orc_rmat_edges(uint32_t scale, double a, double b, double c, uint64_t seed,
                    uint64_t first, uint64_t count, uint32_t *src, uint32_t *dst);
void orc_rmat_weights(uint64_t seed, uint64_t first, uint64_t count, float *w);
/* Count-sort build of CSR (key = src, lists sorted by dst) when by_dst = 0,
 * or CSC (key = dst, lists sorted by src) when by_dst = 1.  adj gets the
 * other endpoint, adj_w (may be NULL) the weight. */
void orc_build_csr(uint32_t V, uint32_t E, const uint32_t *src, const uint32_t *dst, const float *w,
                   int by_dst, uint32_t *off, uint32_t *adj, float *adj_w);

/* ---- fixed point and quantisation (project formats, unpinned) ----------- */

uint64_t orc_fx64_from_double(double x);      /* Q32.32, truncating */
double orc_fx64_to_double(uint64_t f);
uint64_t orc_fx64_mul(uint64_t a, uint64_t b); /* (a*b) >> 32 on 128 bits */
uint32_t orc_fx32_from_float(float x);        /* Q16.16, truncating, saturating */
float orc_fx32_to_float(uint64_t f);
uint32_t orc_fx16_from_float(float x);        /* Q4.12 */
float orc_fx16_to_float(uint64_t f);
uint32_t orc_fx8_from_float(float x);         /* Q2.6 */
float orc_fx8_to_float(uint64_t f);
/* scale = max / (2^bits - 1) as float, 0 when max <= 0 (contributions are
 * non-negative, so zero point 0 covers [0, max]; min is unused) */
float orc_quant_scale(float min, float max, int bits);
/* q = floor(x/scale + 0.5) + zero, clamped to [0, 2^bits - 1] (0 when scale == 0) */
uint32_t orc_quantize(float x, float scale, uint32_t zero, int bits);
/* zero point of the push variant: clamp(round(2^bits - 1 - max/scale)) */
uint32_t orc_quant_zero(float max, float scale, int bits);

/* ---- PageRank ----------------------------------------------------------- */

typedef struct orc_pr_out
{
    uint32_t iterations;   /* reference convention */
    uint32_t active;
    double error_total;
    double rank_sum;
    uint32_t executed;     /* iterations actually run */
} orc_pr_out;

/*
 * PageRank with the reference's semantics for `mode` = the pushpull code
 * (pageRank.c:874-939).  ranks: V floats out (final, divided by V unless
 * init_one_over_n).  Returns 0, or -1 for an unknown mode.
 */
int orc_pagerank(const orc_csr *g, int mode, uint32_t iterations, double epsilon,
                 int init_one_over_n, float *ranks, orc_pr_out *out, int nthreads);

/* Data-driven push (7) / pull-push (8) in the synchronous order (every
 * vertex takes the residual it held when the iteration began); the other
 * end of the range of schedules from orc_pagerank's sequential one. */
void orc_pagerank_dd_sync(const orc_csr *g, int mode, uint32_t iterations, double epsilon, float *ranks);

/* FP64 power iteration, same formulation, exactly `executed` iterations,
 * summing in-edges in CSC order.  ranks: V doubles out. */
void orc_pagerank_f64(const orc_csr *g, uint32_t executed, int init_one_over_n, double *ranks);

/* Personalised PageRank, FP64: r = (1-d) e_seed + d A^T (r / outdeg), from
 * r0 = e_seed, exactly `iterations` pull iterations (dangling mass dropped as
 * in the global variant).  ranks: V doubles out. */
void orc_ppr_f64(const orc_csr *g, uint32_t seed, uint32_t iterations, double damp, double *ranks);
/* The same with a seed set (repeats allowed): each occurrence carries 1/nseeds
 * of the initial rank and of the (1-d) teleport. */
void orc_ppr_f64_multi(const orc_csr *g, const uint32_t *seeds, uint32_t nseeds, uint32_t iterations, double damp,
                       double *ranks);
/* K vectors together in FP32 ([V][K] rows; init[v*K + k] = vector k's
 * starting rank, teleport (1-d) init), OpenMP over vertices (nthreads, 0:
 * all): the CPU timing baseline of the batched GPU form. */
void orc_ppr_f32_batch(const orc_csr *g, uint32_t K, const float *init, uint32_t iterations, float damp,
                       int nthreads, float *ranks);

/* ---- BFS ---------------------------------------------------------------- */

typedef struct orc_bfs_out
{
    uint32_t processed_nodes;  /* reached vertices, source included */
    uint32_t iteration;        /* 1 + frontier steps run */
    uint32_t top_down_steps;
    uint32_t bottom_up_steps;
    uint64_t edges_examined;
    int valid_source;
} orc_bfs_out;

/*
 * BFS with the reference's semantics for `mode` = the pushpull code
 * (BFS.c:241-282).  parents (int32) and distances (uint32) are V-sized
 * outputs initialised as newBFSStatsGraphCSR does (BFS.c:45-81).  `source`
 * is the caller's int; sources above V leave the initial stats.
 * The reference counts the source and the first table row inside printf
 * arguments (`++stats->processed_nodes`, `stats->iteration++`, BFS.c:368,
 * :474, :588, :881); processed_nodes and iteration follow those counts.
 */
void orc_bfs(const orc_csr *g, int mode, int source, int32_t *parents, uint32_t *distances,
             orc_bfs_out *out, int nthreads);

/* ---- SpMV --------------------------------------------------------------- */

/*
 * SpMV with the reference's semantics for `mode` = the pushpull code
 * (SPMV.c:594-620).  x_in may be NULL (reference input vector); x_out and y
 * are V floats out.  checksum = sum of round2(y).
 */
int orc_spmv(const orc_csr *g, int mode, uint32_t iterations, const float *x_in,
             float *x_out, float *y, double *checksum, int nthreads);
/* FP64 y = A^T x (one pull product, weights or 0.0001). */
void orc_spmv_f64(const orc_csr *g, const float *x, double *y);

/* ---- connected components -------------------------------------------- */

/*
 * Every vertex's label is the smallest vertex id of its weakly connected
 * component (edges taken without direction).  The reference's three CSR
 * algorithms (connectedComponents.c:337-720: Shiloach-Vishkin with roots
 * hooked to the lower label and full compression, Afforest with link by the
 * lower id, weakly connected components by atomicMin propagation) all end in
 * this labelling; their iteration counts depend on thread interleaving.
 * orc_cc_min_label: sequential union-find over the out-CSR.
 * orc_cc_sv: the reference's Shiloach-Vishkin loop run serially (hook every
 *   out-edge's higher root to the lower label, compress, repeat while any
 *   hook happened); returns its iteration count.
 * orc_cc_afforest: the reference's CPU Afforest (connectedComponents.c:470-626)
 *   with OpenMP, as the timed CPU baseline: `rounds` neighbour rounds, a
 *   sample of the labels picks the component whose vertices skip the final
 *   link, the final link over the remaining out-edges and (use_in) all
 *   in-edges, compression.  The sample is deterministic (SplitMix64 of
 *   `seed`); any sample gives the same labels.
 */
void orc_cc_min_label(const orc_csr *g, uint32_t *comp);
uint32_t orc_cc_sv(const orc_csr *g, uint32_t *comp);
void orc_cc_afforest(const orc_csr *g, uint32_t rounds, uint32_t samples, uint64_t seed, int use_in,
                     uint32_t *comp, int nthreads);

#ifdef __cplusplus
}
#endif

#endif
