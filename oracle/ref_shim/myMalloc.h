#ifndef SHIM_MYMALLOC_H
#define SHIM_MYMALLOC_H
#include <stdlib.h>
#include <stdio.h>
static inline void *my_malloc(size_t size)
{
    void *p = NULL;
    if (posix_memalign(&p, 64, size ? size : 64) != 0) { fprintf(stderr, "my_malloc failed\n"); exit(1); }
    return p;
}
#endif
