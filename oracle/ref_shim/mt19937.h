#ifndef SHIM_MT19937_H
#define SHIM_MT19937_H
#include <stdint.h>
typedef struct mt19937state { uint32_t mt[624]; int mti; } mt19937state;
#endif
