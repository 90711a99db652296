#ifndef SHIM_GRAPHADJLINKEDLIST_H
#define SHIM_GRAPHADJLINKEDLIST_H
/* Declarations only (never run). */
#include <stdint.h>
struct AdjLinkedListNode { uint32_t dest; float weight; struct AdjLinkedListNode *next; };
struct AdjLinkedList
{
    uint32_t out_degree; uint32_t in_degree; uint8_t visited;
    struct AdjLinkedListNode *outNodes; struct AdjLinkedListNode *inNodes;
};
struct GraphAdjLinkedList { uint32_t num_edges; uint32_t num_vertices; float max_weight; struct AdjLinkedList *vertices; };
#endif
