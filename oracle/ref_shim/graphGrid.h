#ifndef SHIM_GRAPHGRID_H
#define SHIM_GRAPHGRID_H
/* Declarations only: the Grid code of the reference files must compile but
 * is never run. */
#include <stdint.h>
#include "graphCSR.h"
#include "arrayQueue.h"
#include "bitmap.h"
struct Partition { uint32_t num_edges; uint32_t num_vertices; struct EdgeList *edgeList; };
struct Grid
{
    uint32_t num_edges; uint32_t num_vertices; uint32_t num_partitions;
    struct Partition *partitions;
    uint32_t *activePartitions;
    struct Bitmap *activePartitionsMap;
    uint32_t *out_degree;
    uint32_t *in_degree;
};
struct GraphGrid { uint32_t num_edges; uint32_t num_vertices; float max_weight; struct Grid *grid; };
void graphGridReset(struct GraphGrid *graph);
void graphGridSetActivePartitions(struct Grid *grid, uint32_t vertex);
void graphGridSetActivePartitionsMap(struct Grid *grid, uint32_t vertex);
void graphGridResetActivePartitions(struct Grid *grid);
void graphGridResetActivePartitionsMap(struct Grid *grid);
#endif
