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

NOA_HD double pprod_argmin_exact(double K, double q, const noa_dcs_consts &c) {
    const double gamma = x_add(1., x_div(K, c.mass));
    const double x0 = x_div(4. * ME, q);
    const double x1 = x_div(6., x_mul(gamma, x_sub(gamma, x_div(q, c.mass))));
    return x_div(x_add(x0, x_mul(x_mul(2., x_sub(1., x0)), x1)),
                 x_add(1., x_mul(x_sub(1., x1), x_sqrt(x_sub(1., x0)))));
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
