#ifndef ARRAYQUEUE_H
#define ARRAYQUEUE_H

/*
 * Host frontier queue used by the BFS step functions' signatures.
 *
 * The reference takes `struct ArrayQueue` from OpenGraph (absent from the
 * snapshot).  Fields reconstructed from their uses in BFS.c: `head`, `tail`
 * (:725-741, :655), `tail_next` (slideWindowArrayQueue), `queue` (:709),
 * `q_bitmap` / `q_bitmap_next` (:857-880).  The live frontier is
 * queue[head, tail); vertices enqueued during a step land in
 * [tail, tail_next) until slideWindowArrayQueue makes them the frontier.
 */

#include <stdint.h>
#include "bitmap.h"

struct ArrayQueue
{
    uint32_t head;
    uint32_t tail;
    uint32_t tail_next;
    uint32_t size;
    uint32_t *queue;
    struct Bitmap *q_bitmap;
    struct Bitmap *q_bitmap_next;
};

#ifdef __cplusplus
extern "C" {
#endif

struct ArrayQueue *newArrayQueue(uint32_t size);
void freeArrayQueue(struct ArrayQueue *q);
void resetArrayQueue(struct ArrayQueue *q);
void enArrayQueue(struct ArrayQueue *q, uint32_t k);
void enArrayQueueDelayed(struct ArrayQueue *q, uint32_t k);
void slideWindowArrayQueue(struct ArrayQueue *q);
uint32_t sizeArrayQueue(const struct ArrayQueue *q);
int isEmptyArrayQueue(const struct ArrayQueue *q);
void arrayQueueToBitmap(struct ArrayQueue *q, struct Bitmap *b);
void bitmapToArrayQueue(struct Bitmap *b, struct ArrayQueue *q);

#ifdef __cplusplus
}
#endif

#endif
