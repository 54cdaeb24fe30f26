// Floating-point conversions built from integer operations.
//
// GB300's FP64 rate is a small fraction of its FP32 rate, and the double <->
// float conversion instructions run at that rate.  The kernels that narrow
// every element of a vector (vector split, operand preparation) use these exact
// IEEE-754 conversions instead; measured on the tcgen05 engine's FP64-output
// epilogue the hardware widening (float -> double, exact) was faster than
// f32_to_f64, so that epilogue uses the cast:
//   f64_to_f32_rn : round to nearest, ties to even (the rounding of a C cast),
//                   overflow to +-inf, results in the float subnormal range
//                   rounded the same way, NaN -> the canonical quiet NaN;
//   f32_to_f64    : exact widening, subnormal floats normalised.
// Both compile for host and device, so the host tests can check them against
// the CPU's own conversions.
#pragma once
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define VMPS_HD __host__ __device__ __forceinline__
#else
#define VMPS_HD inline
#endif

namespace vmps {

VMPS_HD uint64_t bits_of(double x) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t b;
    memcpy(&b, &x, 8);
    return b;
#endif
}
VMPS_HD uint32_t bits_of(float x) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(x);
#else
    uint32_t b;
    memcpy(&b, &x, 4);
    return b;
#endif
}
VMPS_HD double f64_of(uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)b);
#else
    double x;
    memcpy(&x, &b, 8);
    return x;
#endif
}
VMPS_HD float f32_of(uint32_t b) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(b);
#else
    float x;
    memcpy(&x, &b, 4);
    return x;
#endif
}
VMPS_HD int clz32(uint32_t v) {
#if defined(__CUDA_ARCH__)
    return __clz((int)v);
#else
    return v ? __builtin_clz(v) : 32;
#endif
}

VMPS_HD float f64_to_f32_rn(double x) {
    const uint64_t b = bits_of(x);
    const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
    const int e = (int)((b >> 52) & 0x7FF);
    const uint64_t m = b & 0xFFFFFFFFFFFFFull;
    if (e == 0x7FF) return f32_of(m ? 0x7FFFFFFFu : (sign | 0x7F800000u));
    if (e == 0) return f32_of(sign);   // |x| < 2^-1022: far below half the smallest float subnormal
    const int E = e - 1023;
    if (E > 127) return f32_of(sign | 0x7F800000u);
    if (E >= -126) {
        // normal: keep 23 of the 52 fraction bits; a carry out of the fraction
        // steps the exponent (and reaches +-inf above the largest float)
        const uint32_t keep = (uint32_t)(m >> 29);
        const uint64_t rem = m & ((1ull << 29) - 1), half = 1ull << 28;
        uint32_t r = ((uint32_t)(E + 127) << 23) | keep;
        if (rem > half || (rem == half && (keep & 1u))) r += 1;
        return f32_of(sign | r);
    }
    // float subnormal: q = round(M * 2^(E + 97)) units of 2^-149, M = 2^52 + m
    const int t = -(E + 97);   // right shift, >= 30
    if (t > 53) return f32_of(sign);   // below half the smallest subnormal
    const uint64_t M = (1ull << 52) | m;
    const uint64_t keep = M >> t, rem = M & ((1ull << t) - 1), half = 1ull << (t - 1);
    uint32_t r = (uint32_t)keep;
    if (rem > half || (rem == half && (keep & 1u))) r += 1;   // may become the smallest normal
    return f32_of(sign | r);
}

VMPS_HD double f32_to_f64(float f) {
    const uint32_t b = bits_of(f);
    const uint64_t sign = (uint64_t)(b & 0x80000000u) << 32;
    const uint32_t e = (b >> 23) & 0xFFu, m = b & 0x7FFFFFu;
    if (e == 0xFFu) return f64_of(sign | 0x7FF0000000000000ull | ((uint64_t)m << 29));
    if (e == 0) {
        if (m == 0) return f64_of(sign);
        const int p = 31 - clz32(m);   // top set bit, 0..22: value = 2^(p-149) * (m / 2^p)
        const uint64_t frac = ((uint64_t)m << (52 - p)) & 0xFFFFFFFFFFFFFull;
        return f64_of(sign | ((uint64_t)(p - 149 + 1023) << 52) | frac);
    }
    return f64_of(sign | ((uint64_t)(e - 127 + 1023) << 52) | ((uint64_t)m << 29));
}

}  // namespace vmps
