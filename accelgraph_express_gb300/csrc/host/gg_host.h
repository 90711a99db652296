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

#ifdef __cplusplus
}
#endif

#endif
