// cvt.cuh -- FP32 <-> FP64 conversions on the integer pipes, and division
// by a per-item invariant integer.
//
// This GPU executes 2 FP64 operations per clock per SM, so a conversion on
// the FP64 pipe costs as much as a DFMA of the RK update.  IEEE 754 binary32
// and binary64 differ only in field widths and exponent bias (127 / 1023), so
// for normal numbers both conversions are a few integer operations:
//   f32 -> f64: exact; exponent + 896, mantissa shifted left by 29.
//   f64 -> f32: the top 23 mantissa bits, rounded to nearest with ties to
//               even on the 29 dropped bits by one 64-bit addition; a carry
//               out of the mantissa increments the exponent (and reaches
//               infinity exactly when round-to-nearest overflows).
// Signed zeros are handled inline; subnormal, infinite and NaN inputs, and
// f64 values outside the normal binary32 range, take the hardware conversion.
#pragma once

namespace sgdg {

// The rare inputs go through real calls: a call is not if-converted, so the
// hardware conversion (an FP64-pipe instruction) is not issued, predicated
// off, for every element.
static __device__ __noinline__ double f32_to_f64_rare(float f) { return (double)f; }
static __device__ __noinline__ float f64_to_f32_rare(double x) { return (float)x; }

__device__ __forceinline__ double f32_to_f64(float f) {
    const unsigned u = __float_as_uint(f), a = u & 0x7fffffffu;
    if (a - 0x00800000u >= 0x7f000000u) {                  // biased exponent 0 or 255
        if (a == 0u) return __hiloint2double((int)u, 0);  // a signed zero
        return f32_to_f64_rare(f);                         // subnormal, inf, nan
    }
    // exponent and mantissa move down by 3 bits (11-bit exponent field), the
    // bias grows by 1023 - 127 = 896, the 3 low mantissa bits go to the low word
    return __hiloint2double((int)(((a >> 3) + (896u << 20)) | (u & 0x80000000u)), (int)(u << 29));
}

__device__ __forceinline__ float f64_to_f32(double x) {
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    if ((hi & 0x7fffffffu) - (897u << 20) >= (254u << 20)) {  // |x| < 2^-126, |x| >= 2^128, inf, nan
        if (((hi << 1) | lo) == 0u) return __uint_as_float(hi);  // a signed zero
        return f64_to_f32_rare(x);
    }
    // Round to nearest, ties to even, on the 29 dropped bits: adding one less
    // than half an ulp plus the lowest kept bit carries into the kept bits
    // exactly when rounding goes up (and a carry out of the mantissa raises
    // the exponent, reaching infinity exactly when rounding overflows).
    const unsigned long long b =
        (((unsigned long long)hi << 32) | lo) + (0x0fffffffull + ((lo >> 29) & 1u));
    // Bits 29..60 of the rounded pattern are the 23 kept mantissa bits and
    // the low 9 bits of the exponent; subtracting 896 from that field (mod
    // 2^9, done mod 2^32) leaves the binary32 exponent in bits 23..30 and a
    // zero bit 31, since the exponent is 897..1151 here.
    const unsigned r = (unsigned)(b >> 29) - (896u << 23);
    return __uint_as_float(r | (hi & 0x80000000u));
}

// n / d for 0 <= n < 2^31 and a divisor d >= 1 fixed per work item, with
// (magic, shift) from mf_divisor(): q = floor(n * magic / 2^shift).  This is
// Granlund and Montgomery, "Division by invariant integers using
// multiplication" (PLDI 1994), Theorem 4.2 with N = 31 numerator bits,
// l = ceil(log2 d), magic = floor(2^(31+l) / d) + 1, shift = 31 + l.
__device__ __forceinline__ int div_invariant(int n, unsigned magic, int shift) {
    return (int)(((unsigned long long)(unsigned)n * magic) >> shift);
}

// v / K^p for a compile-time K (each step a multiply by a constant)
template <int K>
__device__ __forceinline__ int div_pow(int v, int p) {
    for (int q = 0; q < p; q++) v /= K;
    return v;
}

}  // namespace sgdg
