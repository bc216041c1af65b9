/*
 * Conversions between double, float and int on the integer pipe.
 *
 * On GB300 the hardware conversions that involve a double (F2F.F32.F64,
 * F2F.F64.F32, I2F.F64) issue to the FP64 pipe and take about one DFMA slot
 * each (measured: a DFMA chain runs at 0.30 ns per iteration per SM, the same
 * chain with a double -> float -> double round trip at 0.87 ns, and with the
 * round trip done by integer operations again at 0.30 ns).  The DCS kernels
 * are FP64-pipe bound, so every conversion on their hot paths goes through
 * these functions instead.  Each one gives exactly the IEEE result of the cast
 * it replaces (round to nearest even, subnormals, signed zeros, infinities;
 * NaNs stay NaNs), using only integer and bit operations.  On the host they
 * are the plain casts.
 */
#pragma once

#if defined(__CUDACC__)
#include <cuda_runtime.h>
#endif

#include <cmath>
#include <cstdint>

#if defined(__CUDACC__)
#define NOA_CONV_HD __host__ __device__ __forceinline__
#else
#define NOA_CONV_HD inline
#endif

namespace fpconv {

// (double)f
NOA_CONV_HD double f64(float f) {
#if defined(__CUDA_ARCH__)
    const unsigned u = __float_as_uint(f);
    const unsigned long long s = (unsigned long long)(u & 0x80000000u) << 32;
    const unsigned a = u & 0x7FFFFFFFu;
    unsigned long long body;
    if (a >= 0x00800000u && a < 0x7F800000u) {
        // normal: move exponent and mantissa up by 29 bits, rebias 127 -> 1023
        body = ((unsigned long long)a << 29) + (896ull << 52);
    } else if (a >= 0x7F800000u) {
        body = 0x7FF0000000000000ull | ((unsigned long long)(a & 0x007FFFFFu) << 29);  // inf / NaN
    } else if (a == 0u) {
        body = 0ull;
    } else {
        // subnormal a * 2^-149: normalise on the highest set bit n
        const int n = 31 - __clz((int)a);
        body = ((unsigned long long)(n + 874) << 52) | (((unsigned long long)a << (52 - n)) & 0x000FFFFFFFFFFFFFull);
    }
    return __longlong_as_double((long long)(s | body));
#else
    return (double)f;
#endif
}

// (float)x, round to nearest even
NOA_CONV_HD float f32(double x) {
#if defined(__CUDA_ARCH__)
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned s = (unsigned)(b >> 32) & 0x80000000u;
    const unsigned long long a = b & 0x7FFFFFFFFFFFFFFFull;
    const unsigned e = (unsigned)(b >> 52) & 0x7FFu;
    unsigned r;
    if (e >= 897u && e <= 1150u) {
        // normal float range: round the 52-bit mantissa to 23 bits (half to even);
        // a carry into the exponent (up to infinity) is the correct result
        const unsigned long long t = a + 0x0FFFFFFFull + ((a >> 29) & 1ull);
        r = (unsigned)(t >> 29) - (896u << 23);
    } else if (e > 1150u) {
        r = (e == 2047u && (a & 0x000FFFFFFFFFFFFFull)) ? 0x7FC00000u : 0x7F800000u;  // NaN / overflow
    } else {
        // float subnormal or zero: shift the significand to units of 2^-149.
        // The shift is clamped to [30, 63] so that no shift is ever out of
        // range, even where the compiler evaluates this branch speculatively
        // (an out-of-range shift is undefined and can poison the selects);
        // a shift of 63 leaves 0, the correct result below 2^-150.
        const unsigned sh = e >= 897u ? 30u : (926u - e > 63u ? 63u : 926u - e);
        const unsigned long long m = (a & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull;
        const unsigned long long q = m >> sh;
        const unsigned long long rem = m & ((1ull << sh) - 1ull);
        const unsigned long long half = 1ull << (sh - 1u);
        r = (unsigned)q + ((rem > half || (rem == half && (q & 1ull))) ? 1u : 0u);
    }
    return __uint_as_float(s | r);
#else
    return (float)x;
#endif
}

// (float)x, round to nearest even, for |x| in the normal float range
// (exponent 2^-126 .. 2^127; a carry to infinity is the correct result);
// NaN for every other input (zero, float subnormals, overflow, inf, NaN).
// Equal to f32 wherever it is not NaN, at a third of its integer
// operations: for tests that send out-of-range inputs to an exact path.
NOA_CONV_HD float f32_normal(double x) {
#if defined(__CUDA_ARCH__)
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned e = (unsigned)(b >> 52) & 0x7FFu;
    const unsigned long long a = b & 0x7FFFFFFFFFFFFFFFull;
    const unsigned long long t = a + 0x0FFFFFFFull + ((a >> 29) & 1ull);
    const unsigned r = ((unsigned)(b >> 32) & 0x80000000u) | ((unsigned)(t >> 29) - (896u << 23));
    return e - 897u <= 253u ? __uint_as_float(r) : __uint_as_float(0x7FC00000u);
#else
    const float f = (float)x;
    return (std::fabs(x) >= 0x1p-126 && std::fabs(x) < 0x1p128) ? f : NAN;
#endif
}

// (double)i
NOA_CONV_HD double f64i(int i) {
#if defined(__CUDA_ARCH__)
    if (i == 0)
        return 0.0;
    const unsigned long long s = i < 0 ? 0x8000000000000000ull : 0ull;
    const unsigned m = i < 0 ? (unsigned)(-(long long)i) : (unsigned)i;
    const int n = 31 - __clz((int)m);  // m < 2^32; __clz of 0x80000000 is 0
    const unsigned long long frac = ((unsigned long long)m << (52 - n)) & 0x000FFFFFFFFFFFFFull;
    return __longlong_as_double((long long)(s | ((unsigned long long)(n + 1023) << 52) | frac));
#else
    return (double)i;
#endif
}

} // namespace fpconv
