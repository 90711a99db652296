#ifndef SHIM_REORDER_H
#define SHIM_REORDER_H
#include <stdint.h>
/* OpenGraph's sort of (degree, id) pairs by ascending degree, in place; the
 * ids come back (the same array) */
uint32_t *radixSortEdgesByDegree(uint32_t *degrees, uint32_t *edges, uint32_t num_edges);
#endif
