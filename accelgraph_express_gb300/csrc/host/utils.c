/*
 * Host utilities named by the drop-in headers: Bitmap and ArrayQueue (whose
 * reference definitions live in the absent OpenGraph submodule), the
 * Mersenne-Twister seeding of struct Arguments, argument defaults, and the
 * PageRank helper functions the reference exports from pageRank.c
 * (addAtomic*, setAtomic :188-252; worklist helpers).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

#include "graphConfig.h"
#include "bitmap.h"
#include "arrayQueue.h"
#include "pageRank.h"

/* ---- Bitmap ------------------------------------------------------------------ */

struct Bitmap *newBitmap(uint32_t size)
{
    struct Bitmap *b = (struct Bitmap *)calloc(1, sizeof(struct Bitmap));
    if (!b) return NULL;
    b->size = size;
    b->bitarray = (uint32_t *)calloc((size_t)(size + 31) / 32 + 1, sizeof(uint32_t));
    if (!b->bitarray) { free(b); return NULL; }
    return b;
}
void freeBitmap(struct Bitmap *b)
{
    if (!b) return;
    free(b->bitarray);
    free(b);
}
void clearBitmap(struct Bitmap *b)
{
    memset(b->bitarray, 0, ((size_t)(b->size + 31) / 32 + 1) * sizeof(uint32_t));
    b->numSetBits = 0;
}
void setBit(struct Bitmap *b, uint32_t pos) { b->bitarray[pos >> 5] |= 1u << (pos & 31); }
void setBitAtomic(struct Bitmap *b, uint32_t pos) { __sync_fetch_and_or(&b->bitarray[pos >> 5], 1u << (pos & 31)); }
uint32_t getBit(const struct Bitmap *b, uint32_t pos) { return (b->bitarray[pos >> 5] >> (pos & 31)) & 1u; }
uint32_t getNumOfSetBits(const struct Bitmap *b)
{
    uint32_t n = 0;
    for (uint32_t i = 0; i < (b->size + 31) / 32; i++) n += (uint32_t)__builtin_popcount(b->bitarray[i]);
    return n;
}
void swapBitmaps(struct Bitmap **a, struct Bitmap **b)
{
    struct Bitmap *t = *a;
    *a = *b;
    *b = t;
}

/* ---- ArrayQueue --------------------------------------------------------------- */

struct ArrayQueue *newArrayQueue(uint32_t size)
{
    struct ArrayQueue *q = (struct ArrayQueue *)calloc(1, sizeof(struct ArrayQueue));
    if (!q) return NULL;
    q->size = size;
    q->queue = (uint32_t *)calloc((size_t)size + 1, sizeof(uint32_t));
    q->q_bitmap = newBitmap(size);
    q->q_bitmap_next = newBitmap(size);
    if (!q->queue || !q->q_bitmap || !q->q_bitmap_next) { freeArrayQueue(q); return NULL; }
    return q;
}
void freeArrayQueue(struct ArrayQueue *q)
{
    if (!q) return;
    freeBitmap(q->q_bitmap);
    freeBitmap(q->q_bitmap_next);
    free(q->queue);
    free(q);
}
void resetArrayQueue(struct ArrayQueue *q) { q->head = q->tail = q->tail_next = 0; }
void enArrayQueue(struct ArrayQueue *q, uint32_t k)
{
    q->queue[q->tail] = k;
    q->tail++;
    q->tail_next = q->tail;
}
void enArrayQueueDelayed(struct ArrayQueue *q, uint32_t k) { q->queue[q->tail_next++] = k; }
void slideWindowArrayQueue(struct ArrayQueue *q)
{
    q->head = q->tail;
    q->tail = q->tail_next;
}
uint32_t sizeArrayQueue(const struct ArrayQueue *q) { return q->tail - q->head; }
int isEmptyArrayQueue(const struct ArrayQueue *q) { return q->head == q->tail; }
void arrayQueueToBitmap(struct ArrayQueue *q, struct Bitmap *b)
{
    for (uint32_t i = q->head; i < q->tail; i++) setBit(b, q->queue[i]);
    b->numSetBits = q->tail - q->head;
}
void bitmapToArrayQueue(struct Bitmap *b, struct ArrayQueue *q)
{
    resetArrayQueue(q);
    for (uint32_t v = 0; v < b->size; v++)
        if (getBit(b, v)) q->queue[q->tail_next++] = v;
    slideWindowArrayQueue(q);
}

/* ---- MT19937 (Matsumoto & Nishimura 1998) -------------------------------------- */

void initializeMersenneState(mt19937state *s, uint32_t seed)
{
    s->mt[0] = seed;
    for (int i = 1; i < MT19937_N; i++)
        s->mt[i] = 1812433253u * (s->mt[i - 1] ^ (s->mt[i - 1] >> 30)) + (uint32_t)i;
    s->mti = MT19937_N;
}

uint32_t generateRandInt(mt19937state *s)
{
    static const uint32_t mag01[2] = {0x0u, 0x9908b0dfu};
    uint32_t y;
    if (s->mti >= MT19937_N)
    {
        int k;
        for (k = 0; k < MT19937_N - 397; k++)
        {
            y = (s->mt[k] & 0x80000000u) | (s->mt[k + 1] & 0x7fffffffu);
            s->mt[k] = s->mt[k + 397] ^ (y >> 1) ^ mag01[y & 1u];
        }
        for (; k < MT19937_N - 1; k++)
        {
            y = (s->mt[k] & 0x80000000u) | (s->mt[k + 1] & 0x7fffffffu);
            s->mt[k] = s->mt[k + (397 - MT19937_N)] ^ (y >> 1) ^ mag01[y & 1u];
        }
        y = (s->mt[MT19937_N - 1] & 0x80000000u) | (s->mt[0] & 0x7fffffffu);
        s->mt[MT19937_N - 1] = s->mt[396] ^ (y >> 1) ^ mag01[y & 1u];
        s->mti = 0;
    }
    y = s->mt[s->mti++];
    y ^= (y >> 11);
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= (y >> 18);
    return y;
}

/* ---- Arguments ------------------------------------------------------------------ */

void argumentsSetDefaults(struct Arguments *a)
{
    memset(a, 0, sizeof(*a));
    a->binSize = 512;
    a->iterations = 20;
    a->trials = 1;
    a->epsilon = 0.0001;
    a->cache_size = 32768;
    a->delta = 1;
    a->pre_numThreads = omp_get_max_threads();
    a->algo_numThreads = omp_get_max_threads();
    a->ker_numThreads = a->algo_numThreads;
    a->fnameb_format = 1;
    a->convert_format = 1;
    a->afu_config = a->afu_config_2 = 0x01;
    a->cu_config = a->cu_config_2 = a->cu_config_3 = a->cu_config_4 = 0x01;
    initializeMersenneState(&a->mt19937var, 27491095);
}

/* ---- PageRank helpers (pageRank.c:188-290) ------------------------------------- */

void addAtomicFloat(float *num, float value)
{
    union { float f; uint32_t u; } o, n;
    do
    {
        o.f = *(volatile float *)num;
        n.f = o.f + value;
    } while (!__sync_bool_compare_and_swap((uint32_t *)num, o.u, n.u));
}

void addAtomicDouble(double *num, double value)
{
    union { double f; uint64_t u; } o, n;
    do
    {
        o.f = *(volatile double *)num;
        n.f = o.f + value;
    } while (!__sync_bool_compare_and_swap((uint64_t *)num, o.u, n.u));
}

void setAtomic(uint64_t *num, uint64_t value)
{
    uint64_t o;
    do
    {
        o = *(volatile uint64_t *)num;
    } while (!__sync_bool_compare_and_swap(num, o, value));
}

void addAtomicFixedPoint(uint64_t *num, uint64_t value) { __sync_fetch_and_add(num, value); }

void pageRankPrint(float *ranks, uint32_t n)
{
    for (uint32_t v = 0; v < n; v++) printf("Rank[%u]=%f \n", v, ranks[v]);
}

void swapWorkLists(uint8_t **a, uint8_t **b)
{
    uint8_t *t = *a;
    *a = *b;
    *b = t;
}
void resetWorkList(uint8_t *w, uint32_t size) { memset(w, 0, size); }
void setWorkList(uint8_t *w, uint32_t size) { memset(w, 1, size); }
