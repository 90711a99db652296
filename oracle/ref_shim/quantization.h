#ifndef SHIM_QUANTIZATION_H
#define SHIM_QUANTIZATION_H
/* This project's quantisation (the reference's lives in the missing OpenGraph
 * quantization.h): scale = max / (2^bits - 1), q = floor(x/scale + 0.5) + zero
 * clamped; the push variant uses 8 bits.  Same definitions as the oracle's
 * orc_quant_* functions. */
#include <stdint.h>
#include <math.h>
struct quant_params { float scale; uint32_t zero; float min; float max; };
struct quant_params_32 { float scale; uint32_t zero; float min; float max; };
struct quant_params_16 { float scale; uint32_t zero; float min; float max; };
struct quant_params_8 { float scale; uint32_t zero; float min; float max; };
#define SHIM_MINMAX(P, A, N) do { (P)->min = 0.0f; (P)->max = 0.0f; \
    for (uint32_t i_ = 0; i_ < (N); i_++) { \
        if (i_ == 0 || (A)[i_] < (P)->min) (P)->min = (A)[i_]; \
        if (i_ == 0 || (A)[i_] > (P)->max) (P)->max = (A)[i_]; } } while (0)
static inline void getMinMax(struct quant_params *p, float *a, uint32_t n) { SHIM_MINMAX(p, a, n); }
static inline void getMinMax_32(struct quant_params_32 *p, float *a, uint32_t n) { SHIM_MINMAX(p, a, n); }
static inline void getMinMax_16(struct quant_params_16 *p, float *a, uint32_t n) { SHIM_MINMAX(p, a, n); }
static inline void getMinMax_8(struct quant_params_8 *p, float *a, uint32_t n) { SHIM_MINMAX(p, a, n); }
static inline float shim_scale(float max, int bits)
{
    if (!(max > 0.0f)) return 0.0f;
    return (float)((double)max / (double)((1ull << bits) - 1));
}
static inline uint32_t shim_quantize(float x, float scale, uint32_t zero, int bits)
{
    double maxq = (double)((1ull << bits) - 1);
    if (scale == 0.0f) return zero;
    double t = floor((double)x / (double)scale + 0.5) + (double)zero;
    if (t < 0.0) return 0;
    if (t > maxq) return (uint32_t)maxq;
    return (uint32_t)t;
}
static inline float GetScale(float mn, float mx) { (void)mn; return shim_scale(mx, 8); }
static inline float GetScale_32(float mn, float mx) { (void)mn; return shim_scale(mx, 32); }
static inline float GetScale_16(float mn, float mx) { (void)mn; return shim_scale(mx, 16); }
static inline float GetScale_8(float mn, float mx) { (void)mn; return shim_scale(mx, 8); }
static inline uint32_t GetZeroPoint(float mx, float scale)
{
    if (scale == 0.0f) return 0;
    double t = floor(255.0 - (double)mx / (double)scale + 0.5);
    if (t < 0.0) return 0;
    if (t > 255.0) return 255;
    return (uint32_t)t;
}
static inline uint32_t quantize(float x, float scale, uint32_t zero) { return shim_quantize(x, scale, zero, 8); }
static inline uint32_t quantize_32(float x, float scale, uint32_t zero) { return shim_quantize(x, scale, zero, 32); }
static inline uint32_t quantize_16(float x, float scale, uint32_t zero) { return shim_quantize(x, scale, zero, 16); }
static inline uint32_t quantize_8(float x, float scale, uint32_t zero) { return shim_quantize(x, scale, zero, 8); }
#endif
