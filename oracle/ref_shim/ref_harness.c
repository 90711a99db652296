/* ctypes-facing harness around the reference's own CSR algorithm functions,
 * compiled from the reference sources (oracle/build_ref.sh).  Builds a
 * GraphCSR over caller arrays, runs one reference entry point with one
 * OpenMP thread (deterministic), copies its outputs out.  Test
 * infrastructure only. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>
#include <fcntl.h>
#include <omp.h>
#include "graphCSR.h"
#include "pageRank.h"
#include "BFS.h"
#include "SPMV.h"
#include "connectedComponents.h"
#include "Judy.h"
#include "ref_emu.h"

/* the reference's sample table (connectedComponents.c:44); only its
 * Afforest frees it, so the harness frees it after every call: a later
 * call on a smaller graph would otherwise index counts with old keys */
extern Pvoid_t JArray;

static int g_quiet = 1;
void ref_set_quiet(int q) { g_quiet = q; }

typedef struct owned
{
    struct GraphCSR g;
    struct Vertex out_v, in_v;
    struct EdgeList out_e, in_e;
    uint32_t *buf[8];
} owned;

static void build(owned *o, uint32_t V, uint32_t E, const uint32_t *out_off, const uint32_t *out_adj,
                  const float *out_w, const uint32_t *in_off, const uint32_t *in_adj, const float *in_w)
{
    memset(o, 0, sizeof(*o));
    uint32_t *odeg = calloc((size_t)V + 1, 4), *ideg = calloc((size_t)V + 1, 4);
    uint32_t *osrc = calloc((size_t)E + 1, 4), *isrc = calloc((size_t)E + 1, 4);
    uint32_t *lab = calloc((size_t)V + 1, 4), *ilab = calloc((size_t)V + 1, 4);
    for (uint32_t v = 0; v < V; v++)
    {
        odeg[v] = out_off[v + 1] - out_off[v];
        ideg[v] = in_off[v + 1] - in_off[v];
        lab[v] = ilab[v] = v;
        for (uint32_t j = out_off[v]; j < out_off[v + 1]; j++) osrc[j] = v;
        for (uint32_t j = in_off[v]; j < in_off[v + 1]; j++) isrc[j] = v;
    }
    o->out_v.out_degree = odeg; o->out_v.in_degree = ideg; o->out_v.edges_idx = (uint32_t *)out_off;
    o->in_v.out_degree = ideg; o->in_v.in_degree = odeg; o->in_v.edges_idx = (uint32_t *)in_off;
    o->out_e.num_edges = E; o->out_e.num_vertices = V;
    o->out_e.edges_array_src = osrc; o->out_e.edges_array_dest = (uint32_t *)out_adj;
    o->out_e.edges_array_weight = (float *)out_w; o->out_e.label_array = lab; o->out_e.inverse_label_array = ilab;
    o->in_e = o->out_e;
    o->in_e.edges_array_src = isrc; o->in_e.edges_array_dest = (uint32_t *)in_adj;
    o->in_e.edges_array_weight = (float *)in_w;
    o->g.num_edges = E; o->g.num_vertices = V;
    o->g.vertices = &o->out_v; o->g.inverse_vertices = &o->in_v;
    o->g.sorted_edges_array = &o->out_e; o->g.inverse_sorted_edges_array = &o->in_e;
    o->buf[0] = odeg; o->buf[1] = ideg; o->buf[2] = osrc; o->buf[3] = isrc; o->buf[4] = lab; o->buf[5] = ilab;
    ref_emu_set_graph(&o->g);
}
static void release(owned *o) { for (int i = 0; i < 8; i++) free(o->buf[i]); }

static void args_init(struct Arguments *a, uint32_t mode, uint32_t iterations, double epsilon, int source)
{
    memset(a, 0, sizeof(*a));
    a->iterations = iterations; a->epsilon = epsilon; a->source = source; a->pushpull = mode;
    a->algo_numThreads = 1; a->ker_numThreads = 1; a->pre_numThreads = 1;
    a->afu_config = a->afu_config_2 = a->cu_config = a->cu_config_2 = 1;
    a->cu_config_3 = a->cu_config_4 = 1;
}

static int quiet_begin(void)
{
    if (!g_quiet) return -1;
    fflush(stdout);
    int saved = dup(1);
    int devnull = open("/dev/null", O_WRONLY);
    dup2(devnull, 1);
    close(devnull);
    return saved;
}
static void quiet_end(int saved)
{
    if (saved < 0) return;
    fflush(stdout);
    dup2(saved, 1);
    close(saved);
}

int ref_pagerank(int mode, uint32_t V, uint32_t E, const uint32_t *out_off, const uint32_t *out_adj,
                 const uint32_t *in_off, const uint32_t *in_adj, uint32_t iterations, double epsilon,
                 float *ranks, uint32_t *iters_out, double *err_out)
{
    static const int cu[14] = {REF_CU_PR_PULL_F32, REF_CU_PR_PUSH_F32, REF_CU_PR_PULL_U64, REF_CU_NONE,
                               REF_CU_PR_PULL_U32, REF_CU_NONE, REF_CU_NONE, REF_CU_NONE, REF_CU_NONE,
                               REF_CU_PR_PULL_U32, REF_CU_PR_PULL_U16, REF_CU_PR_PULL_U8,
                               REF_CU_PR_PULL_U16, REF_CU_PR_PULL_U8};
    if (mode < 0 || mode > 13) return -1;
    omp_set_num_threads(1);
    owned o;
    build(&o, V, E, out_off, out_adj, NULL, in_off, in_adj, NULL);
    struct Arguments a;
    args_init(&a, (uint32_t)mode, iterations, epsilon, 0);
    ref_emu_cu_kind = cu[mode];
    int saved = quiet_begin();
    struct PageRankStats *s = pageRankGraphCSR(&a, &o.g);
    quiet_end(saved);
    memcpy(ranks, s->pageRanks, (size_t)V * sizeof(float));
    *iters_out = s->iterations;
    *err_out = s->error_total;
    freePageRankStats(s);
    release(&o);
    return 0;
}

int ref_bfs(int mode, uint32_t V, uint32_t E, const uint32_t *out_off, const uint32_t *out_adj,
            const uint32_t *in_off, const uint32_t *in_adj, int source,
            int32_t *parents, uint32_t *distances, uint32_t *processed, uint32_t *iteration,
            int *source_out)
{
    if (mode < 0 || mode > 4) return -1;
    omp_set_num_threads(1);
    owned o;
    build(&o, V, E, out_off, out_adj, NULL, in_off, in_adj, NULL);
    struct Arguments a;
    args_init(&a, (uint32_t)mode, 0, 0.0, source);
    ref_emu_cu_kind = mode == 0 ? REF_CU_BFS_BOTTOM_UP : REF_CU_NONE;
    int saved = quiet_begin();
    struct BFSStats *s = breadthFirstSearchGraphCSR(&a, &o.g);
    quiet_end(saved);
    memcpy(parents, s->parents, (size_t)V * sizeof(int32_t));
    memcpy(distances, s->distances, (size_t)V * sizeof(uint32_t));
    *processed = s->processed_nodes;
    *iteration = s->iteration;
    *source_out = a.source;
    freeBFSStats(s);
    release(&o);
    return 0;
}

int ref_spmv(int mode, uint32_t V, uint32_t E, const uint32_t *out_off, const uint32_t *out_adj,
             const float *out_w, const uint32_t *in_off, const uint32_t *in_adj, const float *in_w,
             uint32_t iterations, float *x, float *y)
{
    if (mode < 0 || mode > 3) return -1;
    omp_set_num_threads(1);
    owned o;
    build(&o, V, E, out_off, out_adj, out_w, in_off, in_adj, in_w);
    struct Arguments a;
    args_init(&a, (uint32_t)mode, iterations, 0.0, 0);
    ref_emu_cu_kind = mode == 0 ? REF_CU_SPMV_PULL_F32 : REF_CU_NONE;
    int saved = quiet_begin();
    struct SPMVStats *s = SPMVGraphCSR(&a, &o.g);
    quiet_end(saved);
    memcpy(x, s->vector_input, (size_t)V * sizeof(float));
    memcpy(y, s->vector_output, (size_t)V * sizeof(float));
    freeSPMVStats(s);
    release(&o);
    return 0;
}

/* frees the reference's sample table after a direct call of its
 * sampleFrequentNode, which leaves its keys there */
void ref_cc_reset(void)
{
    Word_t bytes;
    JSLFA(bytes, JArray);
    (void)bytes;
}

/* connected components through the reference's connectedComponentsGraphCSR:
 * mode (pushpull) 1 Afforest, 2 weakly.  Its Shiloach-Vishkin runs on the
 * FPGA, whose connected-components unit is not emulated, so mode 0 is
 * refused.  The generator starts from the reference CLI's seed (27491095);
 * its state after the call (624 words, then the index) is copied out, and
 * so is what the reference's connectedComponentsVerifyGraphCSR returns for
 * the result. */
int ref_cc(int mode, uint32_t V, uint32_t E, const uint32_t *out_off, const uint32_t *out_adj,
           const uint32_t *in_off, const uint32_t *in_adj, uint32_t *components, uint32_t *counts,
           uint32_t *labels, uint32_t *iterations, uint32_t *neighbor_rounds, uint32_t *mt_out,
           uint32_t *verify_out)
{
    if (mode != 1 && mode != 2) return -1;
    omp_set_num_threads(1);
    owned o;
    build(&o, V, E, out_off, out_adj, NULL, in_off, in_adj, NULL);
    struct Arguments a;
    args_init(&a, (uint32_t)mode, 0, 0.0, 0);
    initializeMersenneState(&a.mt19937var, 27491095u);
    ref_emu_cu_kind = REF_CU_NONE;
    int saved = quiet_begin();
    struct CCStats *s = connectedComponentsGraphCSR(&a, &o.g);
    *verify_out = connectedComponentsVerifyGraphCSR(s, &o.g);
    quiet_end(saved);
    Word_t bytes;
    JSLFA(bytes, JArray);
    (void)bytes;
    memcpy(components, s->components, (size_t)V * sizeof(uint32_t));
    memcpy(counts, s->counts, (size_t)V * sizeof(uint32_t));
    memcpy(labels, s->labels, (size_t)V * sizeof(uint32_t));
    *iterations = s->iterations;
    *neighbor_rounds = s->neighbor_rounds;
    memcpy(mt_out, a.mt19937var.mt, sizeof(a.mt19937var.mt));
    mt_out[624] = (uint32_t)a.mt19937var.mti;
    freeCCStats(s);
    release(&o);
    return 0;
}
