/*
 * FP64-accurate elementary functions that issue few FP64 instructions.
 *
 * On GB300 the FP64 pipe retires ~2 DFMA per clock per SM while the FP32 and
 * integer pipes retire 64x more, and CUDA's double-precision log / exp / divide
 * cost about 30 / 16 / 8.5 DFMA-equivalents.  The DCS kernels are bound by
 * exactly those instructions.  The functions here keep double accuracy
 * (a few ulp, checked against CUDA's log/exp/division by tests) but move the
 * range reduction to integer instructions, the table lookups to L1, the
 * initial reciprocal / rsqrt to the MUFU unit, and the high-order polynomial
 * terms -- which are small enough that float precision does not matter -- to
 * FP32:
 *
 *   lean_log   8 FP64 ops.  Table-driven (P. T. P. Tang, ACM TOMS 16(4), 1990):
 *              x = 2^e m, m in [0.707, 1.414); c_t ~ 1/m from the top 8
 *              mantissa bits; r = m c_t - 1 (one FMA, |r| <= 2^-8);
 *              log x = e ln2 - log c_t + log1p(r), log1p by its Taylor series
 *              to r^7, the r^5..r^7 part in FP32.  The two bins next to 1 use
 *              c_t = 1, so log x near 1 keeps full relative accuracy.
 *   lean_exp   7 FP64 ops.  Table-driven (Tang, ACM TOMS 15(2), 1989):
 *              x = (128 k' + j) ln2/128 + r, |r| <= ln2/256; exp x =
 *              2^k' 2^(j/128) exp(r), exp(r) - 1 by its Taylor series to r^5,
 *              the r^4..r^5 part in FP32; 2^k' added to the exponent bits.
 *   lean_rcp   3 FP64 ops.  MUFU reciprocal of float(b), then one
 *              third-order Newton step y (1 + e + e^2), e = 1 - b y.
 *   lean_div   4 FP64 ops: a * lean_rcp(b).
 *   lean_sqrt  6 FP64 ops.  MUFU rsqrt, then two Newton steps on s = x y.
 *
 * Arguments outside the fast range (zero, negative, subnormal, |x| > 700
 * for exp, values outside float range for rcp/sqrt, inf, NaN) take CUDA's
 * IEEE function, so special values behave exactly as in IEEE arithmetic.
 *
 * The counts above are FP64-pipe instructions: the double <-> float and
 * int -> double conversions between the FP64 and FP32 parts go through the
 * integer pipe (fpconv.cuh), because the hardware conversions would occupy
 * the FP64 pipe too.
 */
#pragma once

#include "fpconv.cuh"
#include "lean64_tables.h"

#include <cuda_runtime.h>

namespace lean64 {

__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ float rsqrt_approx(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// x >= 0 finite double compared with a positive constant through the bit
// pattern (integer pipe); NaN compares as larger than every constant.
__device__ __forceinline__ bool bits_ge(double x, double c) {
    return __double_as_longlong(x) >= __double_as_longlong(c);
}

__device__ __forceinline__ double lean_log(double x) {
    const long long b = __double_as_longlong(x);
    // positive, normal and finite?
    if ((unsigned long long)(b - 0x0010000000000000LL) >= 0x7FE0000000000000ULL)
        return log(x);
    const int hi = (int)(b >> 32);
    const int t = (hi >> 12) & 0xFF;
    const int shift = t >= LEAN64_LOG_SPLIT ? 1 : 0;
    const int e = (hi >> 20) - 1023 + shift;
    const double m = __longlong_as_double((b & 0x000FFFFFFFFFFFFFLL) | ((long long)(1023 - shift) << 52));
    const double2 cl = __ldg(&lean64_log_cl[t]);  // {c_t, L_t}, one 16-byte load
    const double c = cl.x, L = cl.y;
    const double r = fma(m, c, -1.0);
    const float rf = fpconv::f32(r);
    const float t5 = fmaf(rf, fmaf(rf, 1.f / 7.f, -1.f / 6.f), 1.f / 5.f);
    const double r2 = r * r;
    double p = fma(r, fpconv::f64(t5), -0.25);
    p = fma(r, p, 1.0 / 3.0);
    p = fma(r, p, -0.5);
    p = fma(r2, p, r);
    return fma(fpconv::f64i(e), LEAN64_LN2, L) + p;
}

__device__ __forceinline__ double lean_exp(double x) {
    if ((__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFLL) >= 0x4085E00000000000LL) // |x| >= 700, inf, NaN
        return exp(x);
    const int k = __float2int_rn(fpconv::f32(x) * (float)LEAN64_INV_LN2N);
    const double kd = fpconv::f64i(k);
    double r = fma(-kd, LEAN64_LN2N_HI, x);
    r = fma(-kd, LEAN64_LN2N_LO, r);
    const float rf = fpconv::f32(r);
    const float t4 = fmaf(rf, 1.f / 120.f, 1.f / 24.f);
    const double r2 = r * r;
    double p = fma(r, fpconv::f64(t4), 1.0 / 6.0);
    p = fma(r, p, 0.5);
    p = fma(r2, p, r);
    const double tj = __ldg(&lean64_exp_t[k & (LEAN64_EXP_N - 1)]);
    const double y = fma(tj, p, tj);
    return __longlong_as_double(
        (long long)((unsigned long long)__double_as_longlong(y) + ((unsigned long long)(long long)(k >> 7) << 52)));
}

__device__ __forceinline__ double lean_rcp(double b) {
    const float bf = fpconv::f32(b);
    const float af = fabsf(bf);
    if (!(af >= 2e-38f && af <= 8e37f))  // 1/b must be a normal float too (the MUFU result is flushed)
        return 1.0 / b;
    const double y = fpconv::f64(rcp_approx(bf));
    double e = fma(-b, y, 1.0);
    e = fma(e, e, e);
    return fma(y, e, y);
}

__device__ __forceinline__ double lean_div(double a, double b) { return a * lean_rcp(b); }

__device__ __forceinline__ double lean_sqrt(double x) {
    const float xf = fpconv::f32(x);
    if (!(xf >= 2e-38f && xf <= 1e38f))
        return sqrt(x);
    const double y = fpconv::f64(rsqrt_approx(xf));
    const double h = 0.5 * y;
    double s = x * y;
    double r = fma(-s, s, x);
    s = fma(r, h, s);
    r = fma(-s, s, x);
    return fma(r, h, s);
}

} // namespace lean64
