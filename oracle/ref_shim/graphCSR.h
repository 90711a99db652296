#ifndef SHIM_GRAPHCSR_H
#define SHIM_GRAPHCSR_H
/* GraphCSR as the hot path uses it; same layout as the product's
 * include/graphCSR.h (checked by the tests). */
#include <stdint.h>
#include "graphConfig.h"
struct Vertex { uint32_t *out_degree; uint32_t *in_degree; uint32_t *edges_idx; };
struct EdgeList
{
    uint32_t num_edges;
    uint32_t num_vertices;
    float max_weight;
    uint32_t *edges_array_src;
    uint32_t *edges_array_dest;
    float *edges_array_weight;
    uint32_t *label_array;
    uint32_t *inverse_label_array;
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
#define EXTRACT_VALUE(x) (x)
#endif
