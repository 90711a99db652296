#ifndef BITMAP_H
#define BITMAP_H

/*
 * Host bitmap used by the BFS step functions' signatures.
 *
 * The reference takes `struct Bitmap` from OpenGraph (absent from the
 * snapshot); the fields are the ones the hot path reads:
 * `bitmap->size` (BFS.c:1076), `bitmap->numSetBits` (BFS.c:600-613).
 * Bit v lives in word v/32, bit v%32.
 */

#include <stdint.h>

struct Bitmap
{
    uint32_t size;        /* number of bits */
    uint32_t numSetBits;
    uint32_t *bitarray;   /* ceil(size/32) words */
};

#ifdef __cplusplus
extern "C" {
#endif

struct Bitmap *newBitmap(uint32_t size);
void freeBitmap(struct Bitmap *bitmap);
void clearBitmap(struct Bitmap *bitmap);
void setBit(struct Bitmap *bitmap, uint32_t pos);
void setBitAtomic(struct Bitmap *bitmap, uint32_t pos);
uint32_t getBit(const struct Bitmap *bitmap, uint32_t pos);
uint32_t getNumOfSetBits(const struct Bitmap *bitmap);
void swapBitmaps(struct Bitmap **bitmap1, struct Bitmap **bitmap2);

#ifdef __cplusplus
}
#endif

#endif
