/* Software stand-in for the reference's CAPI offload (capienv.c) and the
 * FPGA compute units behind it, so the reference's CAPI-offloaded CSR
 * functions run on the CPU.  The CU behaviour is restated from the RTL:
 *   PageRank pull  : next[v] = sum of aux1[u] over in-edges, CSC order
 *                    (cu_PageRank/CSR/PULL/{FloatPoint,FixedPoint,Quantized}/cu/cu_sum_kernel_control.sv)
 *   PageRank push  : next[dst] += aux1[src] over out-edges
 *                    (cu_PageRank/CSR/PUSH/.../cu_sum_kernel_control.sv)
 *   BFS bottom-up  : unvisited v with in-degree > 0 takes the first
 *                    in-neighbour whose workListCurr byte is set
 *                    (cu_BFS/CSR/PULL/BottomUp/cu/cu_update_kernel_control.sv:166-190)
 *   SpMV pull      : y[v] = sum of w*x[u] over in-edges
 * The harness selects the CU ("bitstream") before each call.  Test
 * infrastructure only. */
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#include "graphCSR.h"
#include "libcxl.h"
#include "capienv.h"
#include "ref_emu.h"

int ref_emu_cu_kind = REF_CU_NONE;
static struct WEDGraphCSR *g_wed;
static struct GraphCSR *g_graph;

void ref_emu_set_graph(struct GraphCSR *graph) { g_graph = graph; }

struct WEDGraphCSR *mapGraphCSRToWED(struct GraphCSR *graph)
{
    struct WEDGraphCSR *wed = (struct WEDGraphCSR *)calloc(1, sizeof(struct WEDGraphCSR));
    wed->num_edges = graph->num_edges;
    wed->num_vertices = graph->num_vertices;
    wed->vertex_out_degree = graph->vertices->out_degree;
    wed->vertex_in_degree = graph->vertices->in_degree;
    wed->vertex_edges_idx = graph->vertices->edges_idx;
    wed->edges_array_src = graph->sorted_edges_array->edges_array_src;
    wed->edges_array_dest = graph->sorted_edges_array->edges_array_dest;
    wed->inverse_vertex_out_degree = graph->inverse_vertices->out_degree;
    wed->inverse_vertex_in_degree = graph->inverse_vertices->in_degree;
    wed->inverse_vertex_edges_idx = graph->inverse_vertices->edges_idx;
    wed->inverse_edges_array_src = graph->inverse_sorted_edges_array->edges_array_src;
    wed->inverse_edges_array_dest = graph->inverse_sorted_edges_array->edges_array_dest;
    g_graph = graph;
    return wed;
}
int setupAFUGraphCSR(struct cxl_afu_h **afu, struct WEDGraphCSR *wed) { (void)afu; g_wed = wed; return 0; }
void startAFU(struct cxl_afu_h **afu, struct AFUStatus *s) { (void)afu; (void)s; }
void releaseAFU(struct cxl_afu_h **afu) { (void)afu; g_wed = NULL; }
void waitAFU(struct cxl_afu_h **afu, struct AFUStatus *s) { (void)afu; (void)s; }

void startCU(struct cxl_afu_h **afu, struct AFUStatus *s)
{
    (void)afu;
    const struct GraphCSR *g = g_graph;
    const uint32_t V = g->num_vertices;
    const uint32_t *ioff = g->inverse_vertices->edges_idx;
    const uint32_t *ideg = g->inverse_vertices->out_degree;
    const uint32_t *iadj = g->inverse_sorted_edges_array->edges_array_dest;
    const float *iw = g->inverse_sorted_edges_array->edges_array_weight;
    const uint32_t *ooff = g->vertices->edges_idx;
    const uint32_t *odeg = g->vertices->out_degree;
    const uint32_t *oadj = g->sorted_edges_array->edges_array_dest;
    void *aux1 = g_wed->auxiliary1, *aux2 = g_wed->auxiliary2;
    switch (ref_emu_cu_kind)
    {
    case REF_CU_PR_PULL_F32:
        for (uint32_t v = 0; v < V; v++)
        {
            float sum = 0.0f;
            for (uint32_t j = ioff[v]; j < ioff[v] + ideg[v]; j++) sum += ((float *)aux1)[iadj[j]];
            ((float *)aux2)[v] = sum;
        }
        break;
    case REF_CU_PR_PUSH_F32:
        for (uint32_t v = 0; v < V; v++)
            for (uint32_t j = ooff[v]; j < ooff[v] + odeg[v]; j++)
                ((float *)aux2)[oadj[j]] += ((float *)aux1)[v];
        break;
    case REF_CU_PR_PULL_U64:
    case REF_CU_PR_PULL_U32:
    case REF_CU_PR_PULL_U16:
    case REF_CU_PR_PULL_U8:
        for (uint32_t v = 0; v < V; v++)
        {
            uint64_t sum = 0;
            for (uint32_t j = ioff[v]; j < ioff[v] + ideg[v]; j++)
            {
                uint32_t u = iadj[j];
                switch (ref_emu_cu_kind)
                {
                case REF_CU_PR_PULL_U64: sum += ((uint64_t *)aux1)[u]; break;
                case REF_CU_PR_PULL_U32: sum += ((uint32_t *)aux1)[u]; break;
                case REF_CU_PR_PULL_U16: sum += ((uint16_t *)aux1)[u]; break;
                default: sum += ((uint8_t *)aux1)[u]; break;
                }
            }
            ((uint64_t *)aux2)[v] = sum;
        }
        break;
    case REF_CU_BFS_BOTTOM_UP:
    {
        int *parents = (int *)aux1;
        uint8_t *curr = (uint8_t *)(uintptr_t)s->cu_config_3;
        uint8_t *next = (uint8_t *)(uintptr_t)s->cu_config_4;
        uint64_t nf = 0;
        for (uint32_t v = 0; v < V; v++)
        {
            if (parents[v] >= 0 || ideg[v] == 0) continue;
            for (uint32_t j = ioff[v]; j < ioff[v] + ideg[v]; j++)
            {
                uint32_t u = iadj[j];
                if (curr[u]) { parents[v] = (int)u; next[v] = 1; nf++; break; }
            }
        }
        s->cu_return_done_2 = nf;
        break;
    }
    case REF_CU_SPMV_PULL_F32:
        for (uint32_t v = 0; v < V; v++)
        {
            float sum = 0.0f;
            for (uint32_t j = ioff[v]; j < ioff[v] + ideg[v]; j++)
            {
                float w = iw ? iw[j] : 0.0001f;
                sum += w * ((float *)aux1)[iadj[j]];
            }
            ((float *)aux2)[v] = sum;
        }
        break;
    default:
        /* REF_CU_NONE: a bitstream whose output the host code never reads
         * (SPMVPullFixedPointGraphCSR reads a local array the CU is not given) */
        break;
    }
}

void printMMIO_error(uint64_t error) { (void)error; }
void printWEDGraphCSRPointers(struct WEDGraphCSR *wed) { (void)wed; }
void readCmdResponseStats(struct cxl_afu_h **afu, struct CmdResponseStats *c) { (void)afu; memset(c, 0, sizeof(*c)); }
void printBandwidth(uint64_t size, double t, uint64_t rep) { (void)size; (void)t; (void)rep; }
void printCmdResponseStats(struct CmdResponseStats *c) { (void)c; }

/* worklist helpers (OpenGraph worklist.h) */
void swapWorkLists(uint8_t **a, uint8_t **b) { uint8_t *t = *a; *a = *b; *b = t; }
void resetWorkList(uint8_t *w, uint32_t size) { memset(w, 0, size); }
void setWorkList(uint8_t *w, uint32_t size) { memset(w, 1, size); }
