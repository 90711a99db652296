#ifndef SHIM_ARRAYQUEUE_H
#define SHIM_ARRAYQUEUE_H
#include <stdint.h>
#include "bitmap.h"
struct ArrayQueue
{
    uint32_t head, tail, tail_next, size;
    uint32_t *queue;
    struct Bitmap *q_bitmap;
    struct Bitmap *q_bitmap_next;
};
struct ArrayQueue *newArrayQueue(uint32_t size);
void freeArrayQueue(struct ArrayQueue *q);
void resetArrayQueue(struct ArrayQueue *q);
void enArrayQueue(struct ArrayQueue *q, uint32_t k);
void enArrayQueueWithBitmap(struct ArrayQueue *q, uint32_t k);
void softResetArrayQueue(struct ArrayQueue *q);
uint32_t deArrayQueue(struct ArrayQueue *q);
void slideWindowArrayQueue(struct ArrayQueue *q);
uint32_t sizeArrayQueue(struct ArrayQueue *q);
int isEmptyArrayQueue(struct ArrayQueue *q);
int isEnArrayQueued(struct ArrayQueue *q, uint32_t k);
void flushArrayQueueToShared(struct ArrayQueue *local, struct ArrayQueue *shared);
void arrayQueueToBitmap(struct ArrayQueue *q, struct Bitmap *b);
void bitmapToArrayQueue(struct Bitmap *b, struct ArrayQueue *q, struct ArrayQueue **locals);
void arrayQueueGenerateBitmap(struct ArrayQueue *q);
void arrayQueueToBitmapDualOrder(struct ArrayQueue *q, struct Bitmap *b, uint32_t *labels);
void bitmapToArrayQueueDualOrder(struct Bitmap *b, struct ArrayQueue *q, struct ArrayQueue **locals, uint32_t *labels);
#endif
