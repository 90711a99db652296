#ifndef MT19937_H
#define MT19937_H

/*
 * Mersenne-Twister state carried inside `struct Arguments`.
 *
 * The reference embeds an `mt19937state` in `struct Arguments`
 * (02_capi_graph/include/config/graphConfig.h:47) and seeds it with 27491095
 * (02_capi_graph/src/main/accel-graph.c:329).  Its definition lives in the
 * OpenGraph submodule, which is not part of the reference snapshot, so the
 * layout below is the textbook MT19937 state (624 words + index).  The CSR hot
 * path never reads it; it exists so that `struct Arguments` has the
 * reference's field order.
 */

#include <stdint.h>

#define MT19937_N 624

typedef struct mt19937state
{
    uint32_t mt[MT19937_N];
    int mti;
} mt19937state;

#ifdef __cplusplus
extern "C" {
#endif

/* Seed the state (Matsumoto & Nishimura 1998 initialisation). */
void initializeMersenneState(mt19937state *state, uint32_t seed);
/* Next 32-bit output. */
uint32_t generateRandInt(mt19937state *state);

#ifdef __cplusplus
}
#endif

#endif
