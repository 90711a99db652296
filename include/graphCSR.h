#ifndef GRAPHCSR_H
#define GRAPHCSR_H

/*
 * CSR graph as the CSR traversal hot path consumes it.
 *
 * The reference takes `struct GraphCSR` from its OpenGraph submodule, which is
 * empty in the reference snapshot (.gitmodules:1-3).  The fields below are
 * exactly the ones the hot path touches, reconstructed from their uses:
 *   - graph->num_vertices / num_edges           (pageRank.c:1026, BFS.c:555)
 *   - graph->vertices->{out_degree,in_degree,edges_idx}
 *                                               (BFS.c:711-713, capienv.c:409-411)
 *   - graph->inverse_vertices->{...}            (pageRank.c:968, capienv.c:424-426)
 *   - graph->sorted_edges_array->{edges_array_src,edges_array_dest,
 *       edges_array_weight,label_array,inverse_label_array}
 *                                               (BFS.c:301, SPMV.c:790-806, capienv.c:413-419)
 *   - graph->inverse_sorted_edges_array->{...}  (pageRank.c:969, capienv.c:428-434)
 * This makes the drop-in source/API compatible with the reference's
 * algorithm files; binary layout compatibility with OpenGraph cannot be
 * checked because that source is absent.
 *
 * Storage: uint32 vertex ids and uint32 edge offsets (E < 2^32), the layout
 * the GPU kernels read.  `vertices->edges_idx[v]` is the first edge of v in
 * `sorted_edges_array`; `inverse_vertices->edges_idx[v]` is the first in-edge
 * of v in `inverse_sorted_edges_array`, whose `edges_array_dest` holds the
 * in-neighbour (the edge's source).  Adjacency lists are sorted by neighbour
 * id (count sort by source, stable by destination), so every traversal order
 * is deterministic.
 */

#include <stdint.h>
#include "graphConfig.h"

struct Vertex
{
    uint32_t *out_degree;
    uint32_t *in_degree;
    uint32_t *edges_idx;
};

struct EdgeList
{
    uint32_t num_edges;
    uint32_t num_vertices;
    float max_weight;
    uint32_t *edges_array_src;
    uint32_t *edges_array_dest;
    float *edges_array_weight;      /* NULL: unweighted graph */
    uint32_t *label_array;          /* original id -> internal id (identity unless relabelled) */
    uint32_t *inverse_label_array;  /* internal id -> original id */
};

struct GraphCSR
{
    uint32_t num_edges;
    uint32_t num_vertices;
    float max_weight;
    uint32_t avg_degree;
    struct Vertex *vertices;
    struct Vertex *inverse_vertices;
    struct EdgeList *sorted_edges_array;
    struct EdgeList *inverse_sorted_edges_array;
};

/*
 * The reference masks two "heat" bits off neighbour ids when its mask mode
 * (-M) is on (EXTRACT_VALUE, OpenGraph; cf. VERTEX_CACHE_MASK_U32 in
 * cu_PageRank/CSR/PULL/FixedPoint/pkg/globals_cu_pkg.sv:90).  The GPU path
 * runs with mask mode 0, where the macro is the identity.
 */
#define EXTRACT_VALUE(x) (x)

#ifdef __cplusplus
extern "C" {
#endif

/* ---- edge lists ---------------------------------------------------------- */

struct EdgeList *newEdgeList(uint32_t num_edges, uint32_t num_vertices, int weighted);
void freeEdgeList(struct EdgeList *edgeList);

/*
 * Load the reference's binary edge-list formats (04_test_graphs/TEST/...):
 *   .bin  : little-endian uint32 pairs  (src, dst)
 *   .wbin : little-endian uint32 triples (src, dst, weight); the weight word
 *           is read as an integer and stored as float (the fixture files hold
 *           integer weights).
 * Returns NULL on I/O error (message on stderr).  num_vertices = max id + 1.
 */
struct EdgeList *readEdgeListsbin(const char *fname, int weighted);
/* Text form: one "src dst" or "src dst weight" line per edge. */
struct EdgeList *readEdgeListsText(const char *fname, int weighted);

/*
 * Seeded R-MAT edge list (Chakrabarti, Zhan, Faloutsos, SDM 2004): 2^scale
 * vertices, edge_factor * 2^scale directed edges; each edge picks a quadrant
 * per level with probabilities (a, b, c, 1-a-b-c).  Randomness is counter
 * based: draw l of edge i is splitmix64(seed + (i*scale + l + 1) * phi) with
 * phi = 0x9E3779B97F4A7C15, turned into a 53-bit uniform.  Self-loops and
 * duplicates are kept; there is no label permutation.  With `weighted`,
 * edge i gets float weight (splitmix64(weight_seed + (i+1)*phi) >> 40) * 2^-24
 * in [0,1).  `symmetric` appends the reverse of every edge (2E edges).
 */
struct EdgeList *generateRMATEdgeList(uint32_t scale, uint32_t edge_factor,
                                      double a, double b, double c,
                                      uint64_t seed, int weighted, uint64_t weight_seed,
                                      int symmetric);

/*
 * The block-diagonal union of `ngraphs` R-MAT graphs (no counterpart in the
 * reference; it feeds batched runs over many small graphs): graph g has
 * 2^scales[g] vertices, renumbered from vertex_off[g], and is exactly
 * generateRMATEdgeList(scales[g], edge_factor, a, b, c, seed0 + g, 0, 0, 0)
 * shifted by vertex_off[g].  vertex_off (ngraphs + 1 entries) is written;
 * vertex_off[ngraphs] is the total vertex count.  Unweighted.
 */
struct EdgeList *generateRMATBatchEdgeList(uint32_t ngraphs, const uint32_t *scales, uint32_t edge_factor,
                                           double a, double b, double c, uint64_t seed0, uint32_t *vertex_off);

/* ---- CSR ------------------------------------------------------------------ */

/*
 * Build CSR and inverse CSR (CSC) from an edge list with counting sorts:
 * stable by destination, then stable by source (CSR, lists sorted by
 * destination), then stable by destination (CSC, lists sorted by source).
 * The edge list is not modified and may be freed afterwards.  label arrays
 * are the identity.  Host arrays are page-locked for fast upload when a CUDA
 * device is present (graphCSRFree undoes that).
 */
struct GraphCSR *graphCSRFromEdgeList(const struct EdgeList *edgeList);
/* The same GraphCSR, every array identical, with the sorts run on the GPU
 * (gg_graph_build, then the arrays copied back); NULL on failure (no
 * device, id >= num_vertices, out of memory), with the reason printed. */
struct GraphCSR *graphCSRFromEdgeListDevice(const struct EdgeList *edgeList);
/* The GPU build of the edge list relabelled by mode `lmode` (gg_relabel_order:
 * the reference's -l modes 0..10); both sorted edge lists carry the mapping:
 * label_array[original id] = new id, inverse_label_array[new id] = original
 * id (the drop-in BFS maps its source through label_array, as the reference
 * does).  NULL on failure, with the reason printed. */
struct GraphCSR *graphCSRFromEdgeListRelabelDevice(const struct EdgeList *edgeList, uint32_t lmode, uint64_t seed);
void graphCSRFree(struct GraphCSR *graph);

/* ---- serialisation ----------------------------------------------------------
 * The reference's file options (02_capi_graph/src/main/accel-graph.c): -z
 * picks the input format (:51: 0 text edge list, 1 binary edge list,
 * 2 graphCSR binary), -c the output format of -x serialisation (:115-128,
 * same codes), and -x writes the converted file instead of running an
 * algorithm (:339-341).  The graphCSR binary layout is OpenGraph's, whose
 * code is absent; this one is the project's own: a 32-byte header (magic
 * "AGXCSR1", V, E, weighted, avg_degree, max_weight), then the uint32/float
 * arrays of both Vertex structs (out_degree, in_degree, edges_idx) and both
 * sorted edge lists (src, dest, weight if weighted, label_array,
 * inverse_label_array), forward direction first.  Every function returns 0
 * (or a pointer) on success and -1 (or NULL) with a message on stderr. */
int writeEdgeListsText(const struct EdgeList *edgeList, const char *fname);
/* uint32 pairs, or triples when weighted; the weight word holds the weight
 * rounded to an integer, as the reference's .wbin files and
 * readEdgeListsbin have it. */
int writeEdgeListsbin(const struct EdgeList *edgeList, const char *fname);
int writeGraphCSRbin(const struct GraphCSR *graph, const char *fname);
struct GraphCSR *readGraphCSRbin(const char *fname);
/* The edges of a CSR, in CSR order, under their original ids. */
struct EdgeList *edgeListFromGraphCSR(const struct GraphCSR *graph);
/* Load a graph in format 0 (text), 1 (binary edge list) or 2 (graphCSR
 * binary): the -f / -z pair. */
struct GraphCSR *graphCSRFromFile(const char *fname, uint32_t format, int weighted);
/* -x: read arguments->fnameb in arguments->fnameb_format and write it in
 * arguments->convert_format (weighted when arguments->weighted) to
 * fnameb + ".txt", ".bin" / ".wbin" or ".csr" (accel-graph.c:341). */
void writeSerializedGraphDataStructure(struct Arguments *arguments);

#ifdef __cplusplus
}
#endif

#endif
