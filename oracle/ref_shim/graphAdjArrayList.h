#ifndef SHIM_GRAPHADJARRAYLIST_H
#define SHIM_GRAPHADJARRAYLIST_H
/* Declarations only (never run). */
#include <stdint.h>
#include "graphCSR.h"
struct AdjArrayList
{
    uint32_t out_degree; uint32_t in_degree; uint8_t visited;
    struct EdgeList *outNodes; struct EdgeList *inNodes;
};
struct GraphAdjArrayList { uint32_t num_edges; uint32_t num_vertices; float max_weight; struct AdjArrayList *vertices; };
#endif
