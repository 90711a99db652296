#ifndef SHIM_FIXEDPOINT_H
#define SHIM_FIXEDPOINT_H
/* This project's fixed-point formats (the reference's live in the missing
 * OpenGraph fixedPoint.h): Q32.32 for 64-bit, Q16.16 for 32-bit, Q4.12 for
 * 16-bit, Q2.6 for 8-bit; truncating and saturating.  Same definitions as
 * the oracle's orc_fx* functions. */
#include <stdint.h>
static inline uint64_t DoubleToFixed64(double x)
{
    double t = x * 4294967296.0;
    if (!(t > 0.0)) return 0;
    if (t >= 18446744073709551615.0) return UINT64_MAX;
    return (uint64_t)t;
}
static inline uint64_t FloatToFixed64(float x) { return DoubleToFixed64((double)x); }
static inline uint64_t DoubleToFixed(double x) { return DoubleToFixed64(x); }
static inline uint64_t FloatToFixed(float x) { return DoubleToFixed64((double)x); }
static inline double Fixed64ToDouble(uint64_t f) { return (double)f * (1.0 / 4294967296.0); }
static inline uint64_t UInt32ToFixed64(uint32_t x) { return (uint64_t)x << 32; }
static inline uint64_t UInt64ToFixed(uint64_t x) { return x << 32; }
static inline uint64_t MULFixed64V1(uint64_t a, uint64_t b)
{
    unsigned __int128 p = (unsigned __int128)a * (unsigned __int128)b;
    return (uint64_t)(p >> 32);
}
static inline uint64_t DIVFixed64V1(uint64_t a, uint64_t b)
{
    return b ? (uint64_t)(((unsigned __int128)a << 32) / b) : 0;
}
static inline uint32_t shim_fx_from_float(float x, double scale, uint32_t maxv)
{
    double t = (double)x * scale;
    if (!(t > 0.0)) return 0;
    if (t >= (double)maxv) return maxv;
    return (uint32_t)t;
}
static inline uint32_t FloatToFixed32(float x) { return shim_fx_from_float(x, 65536.0, 0xFFFFFFFFu); }
static inline float Fixed32ToFloat(uint64_t f) { return (float)((double)f * (1.0 / 65536.0)); }
static inline uint32_t FloatToFixed16(float x) { return shim_fx_from_float(x, 4096.0, 0xFFFFu); }
static inline float Fixed16ToFloat(uint64_t f) { return (float)((double)f * (1.0 / 4096.0)); }
static inline uint32_t FloatToFixed8(float x) { return shim_fx_from_float(x, 64.0, 0xFFu); }
static inline float Fixed8ToFloat(uint64_t f) { return (float)((double)f * (1.0 / 64.0)); }
#endif
