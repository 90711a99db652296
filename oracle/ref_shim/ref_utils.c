/* This project's implementations of the OpenGraph utilities the reference's
 * CSR algorithm files call (Bitmap, ArrayQueue, MT19937, the degree sort,
 * Grid stubs).  Test infrastructure only. */
#include <stdlib.h>
#include <string.h>
#include "bitmap.h"
#include "arrayQueue.h"
#include "graphGrid.h"
#include "mt19937.h"
#include "reorder.h"

struct Bitmap *newBitmap(uint32_t size)
{
    struct Bitmap *b = (struct Bitmap *)calloc(1, sizeof(struct Bitmap));
    b->size = size;
    b->bitarray = (uint32_t *)calloc((size + 31) / 32 + 1, sizeof(uint32_t));
    return b;
}
void freeBitmap(struct Bitmap *b) { if (b) { free(b->bitarray); free(b); } }
void clearBitmap(struct Bitmap *b) { memset(b->bitarray, 0, ((b->size + 31) / 32 + 1) * sizeof(uint32_t)); b->numSetBits = 0; }
void setBit(struct Bitmap *b, uint32_t pos) { b->bitarray[pos >> 5] |= 1u << (pos & 31); }
void setBitAtomic(struct Bitmap *b, uint32_t pos) { __sync_fetch_and_or(&b->bitarray[pos >> 5], 1u << (pos & 31)); }
uint32_t getBit(struct Bitmap *b, uint32_t pos) { return (b->bitarray[pos >> 5] >> (pos & 31)) & 1u; }
uint32_t getNumOfSetBits(struct Bitmap *b)
{
    uint32_t n = 0;
    for (uint32_t i = 0; i < (b->size + 31) / 32; i++) n += (uint32_t)__builtin_popcount(b->bitarray[i]);
    return n;
}
void swapBitmaps(struct Bitmap **a, struct Bitmap **b) { struct Bitmap *t = *a; *a = *b; *b = t; }

struct ArrayQueue *newArrayQueue(uint32_t size)
{
    struct ArrayQueue *q = (struct ArrayQueue *)calloc(1, sizeof(struct ArrayQueue));
    q->size = size;
    q->queue = (uint32_t *)calloc((size_t)size + 1, sizeof(uint32_t));
    q->q_bitmap = newBitmap(size);
    q->q_bitmap_next = newBitmap(size);
    return q;
}
void freeArrayQueue(struct ArrayQueue *q)
{
    if (!q) return;
    freeBitmap(q->q_bitmap); freeBitmap(q->q_bitmap_next); free(q->queue); free(q);
}
void resetArrayQueue(struct ArrayQueue *q) { q->head = q->tail = q->tail_next = 0; }
/* append and make visible in the current window */
void enArrayQueue(struct ArrayQueue *q, uint32_t k) { q->queue[q->tail] = k; q->tail++; q->tail_next = q->tail; }
uint32_t deArrayQueue(struct ArrayQueue *q) { return q->queue[q->head++]; }
/* next window = entries appended since the last slide */
void slideWindowArrayQueue(struct ArrayQueue *q) { q->head = q->tail; q->tail = q->tail_next; }
uint32_t sizeArrayQueue(struct ArrayQueue *q) { return q->tail - q->head; }
int isEmptyArrayQueue(struct ArrayQueue *q) { return q->head == q->tail; }
int isEnArrayQueued(struct ArrayQueue *q, uint32_t k) { return (int)getBit(q->q_bitmap, k); }
/* move a thread-local queue's window to the shared queue's pending part */
void flushArrayQueueToShared(struct ArrayQueue *local, struct ArrayQueue *shared)
{
    uint32_t n = local->tail - local->head;
    uint32_t at = __sync_fetch_and_add(&shared->tail_next, n);
    memcpy(shared->queue + at, local->queue + local->head, (size_t)n * sizeof(uint32_t));
    resetArrayQueue(local);
}
/* the window's members as bits; the window itself is left as it is */
void arrayQueueToBitmap(struct ArrayQueue *q, struct Bitmap *b)
{
    for (uint32_t i = q->head; i < q->tail; i++) setBitAtomic(b, q->queue[i]);
    b->numSetBits = q->tail - q->head;
}
/* the bitmap's members, ascending, become the whole queue window */
void bitmapToArrayQueue(struct Bitmap *b, struct ArrayQueue *q, struct ArrayQueue **locals)
{
    (void)locals;
    resetArrayQueue(q);
    for (uint32_t v = 0; v < b->size; v++)
        if (getBit(b, v)) q->queue[q->tail_next++] = v;
    slideWindowArrayQueue(q);
}
void arrayQueueGenerateBitmap(struct ArrayQueue *q)
{
    for (uint32_t i = q->head; i < q->tail; i++) setBit(q->q_bitmap, q->queue[i]);
}
void arrayQueueToBitmapDualOrder(struct ArrayQueue *q, struct Bitmap *b, uint32_t *labels)
{
    for (uint32_t i = q->head; i < q->tail; i++) setBitAtomic(b, labels[q->queue[i]]);
}
void bitmapToArrayQueueDualOrder(struct Bitmap *b, struct ArrayQueue *q, struct ArrayQueue **locals, uint32_t *labels)
{
    (void)locals;
    resetArrayQueue(q);
    for (uint32_t v = 0; v < b->size; v++)
        if (getBit(b, v)) q->queue[q->tail_next++] = labels[v];
    slideWindowArrayQueue(q);
}

void enArrayQueueWithBitmap(struct ArrayQueue *q, uint32_t k)
{
    enArrayQueue(q, k);
    setBit(q->q_bitmap, k);
}

/* the window only; the membership bitmap is kept */
void softResetArrayQueue(struct ArrayQueue *q) { q->head = q->tail = q->tail_next = 0; }

/* MT19937 (Matsumoto and Nishimura, ACM TOMACS 8(1), 1998): the 32-bit
 * generator with its published initialisation and tempering constants */
void initializeMersenneState(mt19937state *s, uint32_t seed)
{
    s->mt[0] = seed;
    for (int i = 1; i < 624; i++)
        s->mt[i] = 1812433253u * (s->mt[i - 1] ^ (s->mt[i - 1] >> 30)) + (uint32_t)i;
    s->mti = 624;
}

uint32_t generateRandInt(mt19937state *s)
{
    if (s->mti >= 624)
    {
        for (int k = 0; k < 624; k++)
        {
            const uint32_t y = (s->mt[k] & 0x80000000u) | (s->mt[(k + 1) % 624] & 0x7fffffffu);
            s->mt[k] = s->mt[(k + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
        }
        s->mti = 0;
    }
    uint32_t y = s->mt[s->mti++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

/* stable sort of the (degree, id) pairs by ascending degree (a counting
 * sort: equal degrees keep their order), both arrays rewritten in place */
uint32_t *radixSortEdgesByDegree(uint32_t *degrees, uint32_t *edges, uint32_t n)
{
    uint32_t maxd = 0;
    for (uint32_t i = 0; i < n; i++)
        if (degrees[i] > maxd) maxd = degrees[i];
    uint32_t *start = (uint32_t *)calloc((size_t)maxd + 2, sizeof(uint32_t));
    uint32_t *d2 = (uint32_t *)malloc((size_t)n * sizeof(uint32_t) + 4);
    uint32_t *e2 = (uint32_t *)malloc((size_t)n * sizeof(uint32_t) + 4);
    if (!start || !d2 || !e2)
    {
        free(start);
        free(d2);
        free(e2);
        return edges;
    }
    for (uint32_t i = 0; i < n; i++)
        start[degrees[i] + 1]++;
    for (uint32_t k = 0; k <= maxd; k++)
        start[k + 1] += start[k];
    for (uint32_t i = 0; i < n; i++)
    {
        const uint32_t pos = start[degrees[i]]++;
        d2[pos] = degrees[i];
        e2[pos] = edges[i];
    }
    memcpy(degrees, d2, (size_t)n * sizeof(uint32_t));
    memcpy(edges, e2, (size_t)n * sizeof(uint32_t));
    free(start);
    free(d2);
    free(e2);
    return edges;
}

/* Grid helpers: only referenced by the Grid variants, which are not run. */
void graphGridReset(struct GraphGrid *graph) { (void)graph; }
void graphGridSetActivePartitions(struct Grid *grid, uint32_t vertex) { (void)grid; (void)vertex; }
void graphGridSetActivePartitionsMap(struct Grid *grid, uint32_t vertex) { (void)grid; (void)vertex; }
void graphGridResetActivePartitions(struct Grid *grid) { (void)grid; }
void graphGridResetActivePartitionsMap(struct Grid *grid) { (void)grid; }
