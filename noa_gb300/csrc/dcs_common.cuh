/*
 * Pieces shared by the FP64 and FP32-compensated DCS device code: the
 * reference's kinematic bounds evaluated in its own IEEE arithmetic, and
 * double helpers that map to lean64 on the GPU and to libm on the host (so
 * that the same source can be checked on a CPU).
 *
 * Bounds (each returns exactly the reference's decision, so both precisions
 * produce the reference's zero pattern):
 *   pprod_argmin_exact  argmin of dcs.hh:169-176 (pair production)
 *   photo_window        dcs.hh:357-381 (photonuclear), Q2min / Q2max
 *   brems_below_qe      q < qe_max of physics.hh:133, 142 (bremsstrahlung)
 *   ion_wmax            W_max of dcs.hh:415-419 (ionisation)
 *
 * Float-float arithmetic (FF, ff_*): pairs of floats carrying ~2^-44, used
 * where a quantity needs more than float but FP64 instructions cost too much
 * (argmin, node arguments, W_max): pprod_argmin_ff.
 */
#pragma once

#include "dcs_consts.h"
#include "fpconv.cuh"

#include <math.h>

#if defined(__CUDACC__)
#include "lean64.cuh"
#define NOA_HD __host__ __device__ __forceinline__
#else
#define NOA_HD inline
#endif

namespace noa_dcs {

constexpr double ME = NOA_ELECTRON_MASS;
constexpr double NA = NOA_AVOGADRO_NUMBER;
constexpr double PH_M = 0.931494;
constexpr double PH_MPI = 0.134977;

// IEEE operations that are never fused (device intrinsics; on the host the
// code is compiled with -ffp-contract=off).
NOA_HD double x_div(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __ddiv_rn(a, b);
#else
    return a / b;
#endif
}
NOA_HD double x_mul(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
NOA_HD double x_add(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
NOA_HD double x_sub(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dsub_rn(a, b);
#else
    return a - b;
#endif
}
NOA_HD double x_sqrt(double a) {
#if defined(__CUDA_ARCH__)
    return __dsqrt_rn(a);
#else
    return sqrt(a);
#endif
}

// Double-accuracy elementary functions (lean64 on the GPU).
NOA_HD double d_log(double x) {
#if defined(__CUDA_ARCH__)
    return lean64::lean_log(x);
#else
    return log(x);
#endif
}
NOA_HD double d_exp(double x) {
#if defined(__CUDA_ARCH__)
    return lean64::lean_exp(x);
#else
    return exp(x);
#endif
}
NOA_HD double d_sqrt(double x) {
#if defined(__CUDA_ARCH__)
    return lean64::lean_sqrt(x);
#else
    return sqrt(x);
#endif
}
NOA_HD double d_rcp(double x) {
#if defined(__CUDA_ARCH__)
    return lean64::lean_rcp(x);
#else
    return 1. / x;
#endif
}

// ---------------------------------------------------------------- float-float
// Unevaluated sums h + l of two floats (Dekker / Knuth error-free transforms
// with FMA), ~2^-44 relative over a short expression: double-like accuracy on
// the FP32 pipe.  from() and to_double() take one FP64 instruction each.
struct FF {
    float h, l;
};
NOA_HD FF ff_from(double x) {
    const float h = fpconv::f32(x);
    return FF{h, fpconv::f32(x - fpconv::f64(h))};
}
NOA_HD double ff_to_double(FF a) { return fpconv::f64(a.h) + fpconv::f64(a.l); }
NOA_HD FF ff_norm(float s, float e) {  // |s| >= |e|
    const float h = s + e;
    return FF{h, e - (h - s)};
}
NOA_HD FF ff_add(FF a, FF b) {
    const float s = a.h + b.h;
    const float bb = s - a.h;
    const float e = (a.h - (s - bb)) + (b.h - bb) + (a.l + b.l);
    return ff_norm(s, e);
}
NOA_HD FF ff_add(float a, FF b) { return ff_add(FF{a, 0.f}, b); }
NOA_HD FF ff_neg(FF a) { return FF{-a.h, -a.l}; }
NOA_HD FF ff_mul(FF a, FF b) {
    const float p = a.h * b.h;
    const float e = fmaf(a.h, b.h, -p) + (a.h * b.l + a.l * b.h);
    return ff_norm(p, e);
}
NOA_HD FF ff_mul(float a, FF b) { return ff_mul(FF{a, 0.f}, b); }
NOA_HD FF ff_div(FF a, FF b) {
    const float q1 = a.h / b.h;
    const FF r = ff_add(a, ff_neg(ff_mul(FF{q1, 0.f}, b)));
    return ff_norm(q1, r.h / b.h);
}
NOA_HD FF ff_sqrt(FF a) {
    const float s = sqrtf(a.h);
    const float r = fmaf(-s, s, a.h) + a.l;  // a - s^2, exact to the rounding of a.l
    return ff_norm(s, r / (2.f * s));
}

// The bit pattern of x as a signed integer: positive doubles order as these do.
NOA_HD long long dbits(double x) {
#if defined(__CUDA_ARCH__)
    return __double_as_longlong(x);
#else
    long long b;
    memcpy(&b, &x, sizeof b);
    return b;
#endif
}

// x = h + l to 2^-47 relative: h is x truncated to 24 significant bits and l
// the rest rounded to float.  Integer and FP32 operations only on the device
// (ff_from takes an FP64 subtraction).  Requires 2^-74 <= x < 2^127.
NOA_HD FF ff_split(double x) {
#if defined(__CUDA_ARCH__)
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned e = (unsigned)(b >> 52);
    const float h = __uint_as_float(((unsigned)(b >> 29) & 0x007FFFFFu) | ((e - 896u) << 23));
    const float scale = __uint_as_float((e - 948u) << 23);  // 2^(e - 1075), the weight of bit 0
    return FF{h, __uint2float_rn((unsigned)b & 0x1FFFFFFFu) * scale};
#else
    unsigned long long b;
    memcpy(&b, &x, sizeof b);
    b &= ~0x1FFFFFFFull;
    double t;
    memcpy(&t, &b, sizeof t);
    return FF{(float)t, (float)(x - t)};
#endif
}

NOA_HD double pprod_argmin_exact(double K, double q, const noa_dcs_consts &c) {
    const double gamma = x_add(1., x_div(K, c.mass));
    const double x0 = x_div(4. * ME, q);
    const double x1 = x_div(6., x_mul(gamma, x_sub(gamma, x_div(q, c.mass))));
    return x_div(x_add(x0, x_mul(x_mul(2., x_sub(1., x0)), x1)),
                 x_add(1., x_mul(x_sub(1., x1), x_sqrt(x_sub(1., x0)))));
}

// argmin (dcs.hh:169-176) in float-float: ~2^-44 relative with four FP64
// instructions (the splits) instead of ~25.  For pairs the exact bounds leave
// open (4 me < q < K + m (1 - 0.75 sqrt(e) Z^1/3)).
NOA_HD FF pprod_argmin_ff(double K, double q, const noa_dcs_consts &c) {
    const FF im{c.inv_mass_h, c.inv_mass_l};
    const FF gamma = ff_add(1.f, ff_mul(ff_from(K), im));
    const FF gmq = ff_add(1.f, ff_mul(ff_from(K - q), im));  // gamma - q/m
    const FF x0 = ff_div(ff_from(4. * ME), ff_from(q));
    const FF x1 = ff_div(FF{6.f, 0.f}, ff_mul(gamma, gmq));
    const FF omx0 = ff_add(1.f, ff_neg(x0));
    const FF num = ff_add(x0, ff_mul(ff_mul(2.f, omx0), x1));
    const FF den = ff_add(1.f, ff_mul(ff_add(1.f, ff_neg(x1)), ff_sqrt(omx0)));
    return ff_div(num, den);
}

NOA_HD bool photo_window(double K, double q, const noa_dcs_consts &c, double &Q2min, double &Q2max) {
    if ((q < 1.) || (q < 2E-03 * K))
        return false;
    const double mass = c.mass;
    const double E = K + mass;
    if ((q >= (E - mass)) || (q <= c.ph_q_min))
        return false;
    const double y = x_div(q, E);
    Q2min = x_div(x_mul(x_mul(x_mul(mass, mass), y), y), x_sub(1., y));
    Q2max = x_sub(x_mul(2.0 * PH_M, q - PH_MPI), PH_MPI * PH_MPI);
    if ((Q2max < Q2min) | (Q2min < 0))
        return false;
    return true;
}

NOA_HD bool brems_below_qe(double E, double q, const noa_dcs_consts &c) {
    return q < x_div(E, x_add(1., x_div(c.br_half_m2, x_mul(ME, E))));
}

NOA_HD double ion_wmax(double P2, double E, const noa_dcs_consts &c) {
    return x_div(2. * ME * P2, x_add(x_mul(c.mass, c.mass), x_mul(ME, ME + 2. * E)));
}

} // namespace noa_dcs
