/*
 * Internal helpers of the host side of the drop-in (not part of the ABI).
 */
#ifndef GG_HOST_H
#define GG_HOST_H

#include <stddef.h>
#include <stdint.h>

#include "graphCSR.h"
#include "gg_runtime.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Page-lock host memory for fast upload when a CUDA device is present;
 * silently does nothing otherwise.  gg_host_unpin(p) undoes it (no-op for
 * pointers that were not pinned). */
void gg_host_pin(void *p, size_t bytes);
void gg_host_unpin(void *p);

/* Device mapping of `graph` carrying at least `what`, for one drop-in call:
 * either a fresh mapping (released by gpu_release_call) or the resident one
 * when GraphGpuOptions.keep_resident is set or `force_resident` is 1.
 * Returns NULL after printing the error to stderr. */
gg_graph *gpu_acquire(struct GraphCSR *graph, uint32_t what, int force_resident);
void gpu_release_call(struct GraphCSR *graph, gg_graph *g);
/* record the status of a failed drop-in call and print it */
void gpu_report(const char *where, gg_status st);
const GraphGpuOptions *gpu_options(void);

double gg_seconds(void);

/* Large host arrays of the stats structs, recycled: a freed array of at
 * least 64 KiB is kept (up to 8 arrays, 1 GiB in all) and handed out again
 * for a request of the same size, so a drop-in call repeated on one graph
 * does not fault in fresh pages for its result arrays every time.  take
 * returns memory as malloc does (contents undefined); give takes memory from
 * take or malloc, of the given size. */
void *gg_host_array_take(size_t bytes);
void gg_host_array_give(void *p, size_t bytes);

#ifdef __cplusplus
}
#endif

#endif
