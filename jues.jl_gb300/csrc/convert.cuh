// Exact FP32 -> FP64 conversion on the integer pipes (device code).
#pragma once
#include <cstdint>

namespace jues {

// FP32 -> FP64 on the integer pipes, exact for every input (GB300's FP64 pipe, conversions
// included, runs at about two operations per clock per SM): the exponent is rebiased and the
// significand shifted; subnormals are normalised with a leading-zero count
__device__ __forceinline__ double f32_to_f64(float f) {
    const uint32_t u = __float_as_uint(f), e = (u >> 23) & 0xFFu, m = u & 0x7FFFFFu, s = u & 0x80000000u;
    uint32_t hi, lo;
    if (e - 1u < 254u) {          // normal
        hi = s | ((e + 896u) << 20) | (m >> 3);
        lo = m << 29;
    } else if (e == 0xFFu) {      // infinity, NaN
        hi = s | 0x7FF00000u | (m >> 3);
        lo = m << 29;
    } else if (m == 0u) {         // zero
        hi = s;
        lo = 0u;
    } else {                      // subnormal m 2^-149, leading bit at position b
        const int b = 31 - __clz((int)m);
        const uint64_t mant = ((uint64_t)m << (52 - b)) & 0xFFFFFFFFFFFFFull;
        hi = s | ((uint32_t)(b + 874) << 20) | (uint32_t)(mant >> 32);
        lo = (uint32_t)mant;
    }
    return __hiloint2double((int)hi, (int)lo);
}
// FP32 -> FP64 for a normal number or zero (the exponent rebiased by 1023 - 127 = 896)
__device__ __forceinline__ double f32_to_f64_normal(float f) {
    const uint32_t u = __float_as_uint(f), a = u & 0x7FFFFFFFu;
    const uint32_t hi = (a == 0u ? 0u : (a >> 3) + (896u << 20)) | (u & 0x80000000u);
    return __hiloint2double((int)hi, (int)(u << 29));
}


// the value as FP64 (FP64 inputs unchanged, FP32 through the integer conversion)
__device__ __forceinline__ double to_f64(double x) { return x; }
__device__ __forceinline__ double to_f64(float x) {
    const uint32_t a = __float_as_uint(x) & 0x7FFFFFFFu;
    if (__builtin_expect((a - 1u < 0x7FFFFFu) | (a > 0x7F7FFFFFu), 0)) return f32_to_f64(x);   // subnormal, inf, NaN
    return f32_to_f64_normal(x);
}

}  // namespace jues
