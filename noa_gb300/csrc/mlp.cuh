/*
 * Learned DCS surrogate: shared definitions.
 *
 * A 4 -> 128 -> 128 -> 128 -> 1 SiLU network predicts, for pair production or
 * photonuclear, the residual of log(DCS) over a cheap analytic baseline that
 * carries the kinematic-limit behaviour:
 *
 *   pair production  log DCS = log(c Z (E - q)/(q E) (m + K) N_A/A  (-tmin)) + r
 *                    (dcs.hh:254-257 without zeta, times the length -tmin of
 *                    the t-integral, dcs.hh:176-179)
 *   photonuclear     log DCS = log(cf/q (1 - y + y^2/2) (1/Q2min - 1/Q2max)
 *                                  (m + K) N_A/A) + r
 *                    (the Q2 integral of the leading 1/Q2^2 term of
 *                    dcs.hh:348-354 over the window of dcs.hh:377-381)
 *
 * Features: (log K, log nu, Z/100, log A), nu = q/(K + m), shifted and
 * scaled to about [-1, 1].  Parameters are kept in FP32 (master copy, Adam
 * state); the first and last layers stay FP32, W2 and W3 and the hidden
 * activations enter the tensor-core products as BF16 hi + lo pairs
 * (16 significant bits) with FP32 accumulation.
 *
 * Parameter vector layout (MLP_NPARAM floats):
 *   W1[128][4] b1[128] W2[128][128] b2[128] W3[128][128] b3[128] Wo[128] bo
 */
#pragma once

#include "dcs_fp32c.cuh"
#include "dcs_fp64.cuh"

#include <cuda_bf16.h>

namespace noa_mlp {

constexpr int IN = 4;
constexpr int H = 128;
constexpr int OFF_W1 = 0;
constexpr int OFF_B1 = OFF_W1 + H * IN;
constexpr int OFF_W2 = OFF_B1 + H;
constexpr int OFF_B2 = OFF_W2 + H * H;
constexpr int OFF_W3 = OFF_B2 + H;
constexpr int OFF_B3 = OFF_W3 + H * H;
constexpr int OFF_WO = OFF_B3 + H;
constexpr int OFF_BO = OFF_WO + H;
constexpr int NPARAM = OFF_BO + 1;

// Feature / target normalisation: f = (raw - shift) * scale.
struct Norm {
    float in_shift[IN];
    float in_scale[IN];
    float out_shift;
    float out_scale;  // r = out_shift + y / out_scale
};

// SiLU and its derivative.  On the GPU through the MUFU exponential and an
// approximate division (relative error ~2^-21), in training and inference
// alike; z / (1 + inf) gives the correct limit 0.
__host__ __device__ __forceinline__ float silu(float z) {
#if defined(__CUDA_ARCH__)
    return __fdividef(z, 1.f + __expf(-z));
#else
    return z / (1.f + expf(-z));
#endif
}
__host__ __device__ __forceinline__ float dsilu(float z) {
#if defined(__CUDA_ARCH__)
    const float s = __fdividef(1.f, 1.f + __expf(-z));
#else
    const float s = 1.f / (1.f + expf(-z));
#endif
    return s * (1.f + z * (1.f - s));
}

// Baseline of log DCS and the open / closed decision, in FP64 with the exact
// bounds of the plain kernels.  Returns false for a closed pair (DCS = 0).
template <int PROC>
__device__ __forceinline__ bool baseline(double K, double q, const noa_dcs_consts &c, double &base) {
    using namespace noa_dcs;
    const double mass = c.mass;
    const double E = K + mass;
    if (PROC == NOA_DCS_PAIR_PRODUCTION) {
        if (q <= 4. * ME || q >= K + c.pp_kmax_shift)
            return false;
        const double argmin = pprod_argmin_exact(K, q, c);
        if ((argmin >= 1.) || (argmin <= 0.))
            return false;
        const double tmin = d_log(argmin);
        base = d_log(c.pp_cZ * c.Zd * (E - q) * d_rcp(q * E) * (mass + K) * c.scale_A * (-tmin));
        return true;
    } else {
        double Q2min, Q2max;
        if (!photo_window(K, q, c, Q2min, Q2max))
            return false;
        const double y = q * d_rcp(E);
        const double w = d_rcp(Q2min) - d_rcp(Q2max);
        base = d_log(2.603096E-35 * d_rcp(q) * (1. - y + 0.5 * y * y) * w * (mass + K) * c.scale_A);
        return true;
    }
}

// Inference forms of baseline().
// Float pre-check of the reference's first early returns: true only where
// the pair is certainly closed (margins of 1e-5 relative, far above float
// rounding); the exact checks decide everything else.
template <int PROC>
__device__ __forceinline__ bool surely_closed(double K, double q, const noa_dcs_consts &c) {
    // NaN outside the normal float range: no pair is then "surely closed"
    const float Kf = fpconv::f32_normal(K), qf = fpconv::f32_normal(q);
    if (PROC == NOA_DCS_PAIR_PRODUCTION)
        return qf < (float)(4. * noa_dcs::ME) * 0.99999f || qf > (Kf + c.pp_kmax_shift_f) * 1.00001f;
    return qf < 0.99999f || qf < 2E-03f * Kf * 0.99999f;
}

// The open / closed decision as the FP64 kernels take it: float first, the
// exact IEEE decision near a bound.
template <int PROC>
__device__ __forceinline__ bool open_fast(double K, double q, const noa_dcs_consts &c) {
    if (surely_closed<PROC>(K, q, c))
        return false;
    return PROC == NOA_DCS_PAIR_PRODUCTION ? noa_dcs::pprod_live(K, q, c) : noa_dcs::photo_live(K, q, c);
}

// The baseline of an open pair as a sum of float logs (about 1e-6 absolute,
// far below the surrogate's 1e-3).  False where float cannot form it
// (photonuclear within 1e-4 of its Q2 window closing): the pair then goes to
// the fallback.
template <int PROC>
__device__ __forceinline__ bool baseline_value(double K, double q, const noa_dcs_consts &c, float &base) {
    using namespace noa_dcs;
    const double mass = c.mass;
    const double E = K + mass;
    const float Ef = fpconv::f32(E), qf = fpconv::f32(q), Emq = fpconv::f32(E - q);
    if (PROC == NOA_DCS_PAIR_PRODUCTION) {
        // log(argmin) from the float-float argmin, through log1p near
        // argmin = 1 (where a.h - 1 is exact)
        const FF a = pprod_argmin_ff(K, q, c);
        const float tmin = a.h >= 0.5f ? log1pf((a.h - 1.f) + a.l) : logf(a.h);
        base = logf(fpconv::f32(c.pp_cZ * c.Zd * c.scale_A)) + logf(Emq) - logf(qf) - logf(Ef) +
               logf(fpconv::f32(mass + K)) + logf(-tmin);
        return true;
    } else {
        const float y = qf / Ef, omy = Emq / Ef;
        const float Q2min = fpconv::f32(mass * mass) * y * y / omy;
        const float Q2max = (float)(2.0 * PH_M) * fpconv::f32(q - PH_MPI) - (float)(PH_MPI * PH_MPI);
        if (!(Q2max - Q2min > 1e-4f * fmaxf(fabsf(Q2max), fabsf(Q2min))) || !(Q2min > 0.f))
            return false;
        base = logf(fpconv::f32(2.603096E-35 * c.scale_A)) - logf(qf) + logf(omy + 0.5f * y * y) +
               logf(1.f / Q2min - 1.f / Q2max) + logf(fpconv::f32(mass + K));
        return true;
    }
}

__device__ __forceinline__ void features(double K, double q, double mass, float Zf, float logA, const Norm &n,
                                         float f[IN]) {
    const double nu = q / (K + mass);
    const float raw[IN] = {(float)log(K), (float)log(nu), Zf * 0.01f, logA};
#pragma unroll
    for (int i = 0; i < IN; i++)
        f[i] = (raw[i] - n.in_shift[i]) * n.in_scale[i];
}

} // namespace noa_mlp
