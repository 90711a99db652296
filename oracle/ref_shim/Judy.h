#ifndef SHIM_JUDY_H
#define SHIM_JUDY_H

/* Stand-in for the part of the Judy library (libJudy, linked by the
 * reference's Makefile as -lJudy, no version pinned; not installed here)
 * that the reference's connectedComponents.c uses: the JudyL macros JLI
 * (insert an index, value 0 when new, yield a pointer to its value), JLF
 * (first index >= Index), JLN (next index > Index) and JSLFA (free the
 * whole array, set it to NULL, yield the bytes freed).  A JudyL array maps
 * machine-word indices to machine-word values and is walked in ascending
 * index order; this one is a dense table grown to the largest index
 * inserted, which suits the vertex-id keys of that file.  Test
 * infrastructure only. */

#include <stdlib.h>
#include <string.h>

typedef unsigned long Word_t, *PWord_t;
typedef void *Pvoid_t;

typedef struct
{
    Word_t cap;
    Word_t *val;
    unsigned char *has;
} shim_judyl;

static inline Word_t *shim_judyl_ins(Pvoid_t *pa, Word_t idx)
{
    shim_judyl *a = (shim_judyl *)*pa;
    if (!a)
    {
        a = (shim_judyl *)calloc(1, sizeof(*a));
        if (!a) return NULL;
        *pa = a;
    }
    if (idx >= a->cap)
    {
        Word_t cap = a->cap ? a->cap : 1024;
        while (cap <= idx) cap *= 2;
        Word_t *v = (Word_t *)realloc(a->val, cap * sizeof(Word_t));
        if (!v) return NULL;
        a->val = v;
        unsigned char *h = (unsigned char *)realloc(a->has, cap);
        if (!h) return NULL;
        a->has = h;
        memset(a->val + a->cap, 0, (cap - a->cap) * sizeof(Word_t));
        memset(a->has + a->cap, 0, cap - a->cap);
        a->cap = cap;
    }
    if (!a->has[idx])
    {
        a->has[idx] = 1;
        a->val[idx] = 0;
    }
    return &a->val[idx];
}

static inline Word_t *shim_judyl_first(Pvoid_t pa, Word_t *idx)
{
    shim_judyl *a = (shim_judyl *)pa;
    if (!a) return NULL;
    for (Word_t i = *idx; i < a->cap; i++)
        if (a->has[i])
        {
            *idx = i;
            return &a->val[i];
        }
    return NULL;
}

static inline Word_t *shim_judyl_next(Pvoid_t pa, Word_t *idx)
{
    if (*idx == (Word_t)-1) return NULL;
    Word_t i = *idx + 1;
    Word_t *p = shim_judyl_first(pa, &i);
    if (p) *idx = i;
    return p;
}

static inline Word_t shim_judyl_free(Pvoid_t *pa)
{
    shim_judyl *a = (shim_judyl *)*pa;
    Word_t bytes = 0;
    if (a)
    {
        bytes = a->cap * (sizeof(Word_t) + 1);
        free(a->val);
        free(a->has);
        free(a);
    }
    *pa = NULL;
    return bytes;
}

#define JLI(PValue, PJLArray, Index) ((PValue) = shim_judyl_ins(&(PJLArray), (Word_t)(Index)))
#define JLF(PValue, PJLArray, Index) ((PValue) = shim_judyl_first((PJLArray), &(Index)))
#define JLN(PValue, PJLArray, Index) ((PValue) = shim_judyl_next((PJLArray), &(Index)))
#define JSLFA(Bytes, PJSLArray) ((Bytes) = shim_judyl_free(&(PJSLArray)))

#endif
