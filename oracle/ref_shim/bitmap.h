#ifndef SHIM_BITMAP_H
#define SHIM_BITMAP_H
#include <stdint.h>
#define kBitsPerWord 32 /* bits per bitarray word */
struct Bitmap { uint32_t size; uint32_t numSetBits; uint32_t *bitarray; };
struct Bitmap *newBitmap(uint32_t size);
void freeBitmap(struct Bitmap *b);
void clearBitmap(struct Bitmap *b);
void setBit(struct Bitmap *b, uint32_t pos);
void setBitAtomic(struct Bitmap *b, uint32_t pos);
uint32_t getBit(struct Bitmap *b, uint32_t pos);
uint32_t getNumOfSetBits(struct Bitmap *b);
void swapBitmaps(struct Bitmap **a, struct Bitmap **b);
#endif
