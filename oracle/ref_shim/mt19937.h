#ifndef SHIM_MT19937_H
#define SHIM_MT19937_H
#include <stdint.h>
typedef struct mt19937state { uint32_t mt[624]; int mti; } mt19937state;
void initializeMersenneState(mt19937state *s, uint32_t seed);
uint32_t generateRandInt(mt19937state *s);
#endif
