// cvt.cuh -- FP32 <-> FP64 conversions on the integer pipes, and division
// by a per-item invariant integer.
//
// This GPU executes 2 FP64 operations per clock per SM, so a conversion on
// the FP64 pipe costs as much as a DFMA of the RK update.  IEEE 754 binary32
// and binary64 differ only in field widths and exponent bias (127 / 1023), so
// for normal numbers both conversions are a few shifts and masks:
//   f32 -> f64: exact; exponent + 896, mantissa shifted left by 29.
//   f64 -> f32: the top 23 mantissa bits, rounded to nearest with ties to
//               even on the 29 dropped bits; a carry out of the mantissa
//               increments the exponent (and reaches infinity exactly when
//               round-to-nearest overflows).
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
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    if (e - 1u >= 254u && (u << 1) != 0u) return f32_to_f64_rare(f);  // subnormal, inf, nan
    // normal, or a signed zero (e == 0, mantissa 0)
    const unsigned hi = (u & 0x80000000u) | (e != 0u ? ((e + 896u) << 20) | ((u >> 3) & 0x000fffffu) : 0u);
    return __hiloint2double((int)hi, (int)(u << 29));
}

__device__ __forceinline__ float f64_to_f32(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const unsigned e = (hi >> 20) & 0x7ffu;
    if (e - 897u >= 254u) {                                // |x| < 2^-126, |x| >= 2^128, inf, nan
        if (((hi << 1) | lo) == 0u) return __uint_as_float(hi);  // a signed zero
        return f64_to_f32_rare(x);
    }
    unsigned r = (hi & 0x80000000u) | ((e - 896u) << 23) | ((hi & 0x000fffffu) << 3) | (lo >> 29);
    const unsigned rest = lo & 0x1fffffffu;  // the dropped bits; half an ulp is 2^28
    r += (rest > 0x10000000u ? 1u : 0u) | (rest == 0x10000000u ? (r & 1u) : 0u);
    return __uint_as_float(r);
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
