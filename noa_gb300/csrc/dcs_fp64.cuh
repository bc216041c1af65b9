/*
 * FP64 device functions of the four muon DCS processes.
 *
 *   bremsstrahlung   physics.hh:114-153
 *   pair production  dcs.hh:144-258, 8-node GL numerics.hh:110-129
 *   photonuclear     dcs.hh:261-405, 9-node GL numerics.hh:131-152
 *   ionisation       dcs.hh:408-443
 *
 * Accuracy contract: FP64 -- the reference's own metric (mean relative error,
 * common.hh:228-236) against its CPU output stays below 1e-12.  The formulas
 * are the reference's; what differs is how they are evaluated on a GPU whose
 * FP64 pipe is ~64x slower than its FP32 and integer pipes:
 *
 *  - what depends only on (element, mass) comes precomputed in
 *    noa_dcs_consts (dcs_consts.h), bit-identical to the reference's values;
 *  - log / exp / reciprocal / division inside the quadrature bodies use the
 *    lean64 functions (lean64.cuh): same accuracy class, 1 / 2 / 0 / 1 FP64
 *    instructions instead of CUDA's ~30 / 16 / 8 / 8.5, the rest on the
 *    integer and FP32 pipes; divisions by a shared denominator reuse one
 *    reciprocal;
 *  - branch tests on non-negative doubles compare bit patterns on the
 *    integer pipe (lean64::bits_ge).
 *
 * Every early exit of the reference is decided exactly as the reference
 * decides it: the bound expressions are evaluated in IEEE arithmetic in the
 * reference's order, with __d*_rn intrinsics where the compiler could
 * otherwise fuse a product into an addition.  The zero / non-zero pattern is
 * therefore identical, also for pairs placed exactly on a bound, and NaN
 * inputs propagate as on the CPU.  The `*_live` predicates evaluate only those
 * bounds, so that a kernel can drop closed pairs before the quadrature.
 */
#pragma once

#include "dcs_common.cuh"

namespace noa_dcs {

using lean64::bits_ge;
using lean64::lean_div;
using lean64::lean_exp;
using lean64::lean_log;
using lean64::lean_rcp;

// Gauss-Legendre literals, numerics.hh:116-121 (8 nodes on [0,1]) and
// numerics.hh:137-144 (9 nodes on [-1,1]).  They are the reference's 8-digit
// truncations; the exact nodes would move results by ~5e-9.
__constant__ double kGL8X[8] = {0.01985507, 0.10166676, 0.2372338, 0.40828268,
                                0.59171732, 0.7627662, 0.89833324, 0.98014493};
__constant__ double kGL8W[8] = {0.05061427, 0.11119052, 0.15685332, 0.18134189,
                                0.18134189, 0.15685332, 0.11119052, 0.05061427};
__constant__ double kGL9X[9] = {0.0000000000000000, -0.8360311073266358, 0.8360311073266358,
                                -0.9681602395076261, 0.9681602395076261, -0.3242534234038089,
                                0.3242534234038089, -0.6133714327005904, 0.6133714327005904};
__constant__ double kGL9W[9] = {0.3302393550012598, 0.1806481606948574, 0.1806481606948574,
                                0.0812743883615744, 0.0812743883615744, 0.3123470770400029,
                                0.3123470770400029, 0.2606106964029354, 0.2606106964029354};

// Clamp of the reference's `if (v < 0.) v = 0.;` that keeps NaN.
__device__ __forceinline__ double clamp0(double v) {
    const long long b = __double_as_longlong(v);
    return (b < 0 && (b & 0x7FFFFFFFFFFFFFFFLL) <= 0x7FF0000000000000LL) ? 0. : v;
}

// Out-of-line copies of the lean64 functions for the two quadrature bodies.
// Inlined, every call site adds ~100 integer and FP32 instructions; the
// photonuclear node (17 transcendental calls) then outgrows the instruction
// cache (ncu: 11.7 "no instruction" stalls per issue) and runs at 87 ms per
// 1e8 pairs against 50 ms with these calls; pair production gains 9%.
// Bremsstrahlung and ionisation, with a few calls each, keep them inlined.
static __device__ __noinline__ double ol_log(double x) { return lean_log(x); }
static __device__ __noinline__ double ol_exp(double x) { return lean_exp(x); }
static __device__ __noinline__ double ol_rcp(double x) { return lean_rcp(x); }
static __device__ __noinline__ double ol_div(double a, double b) { return lean_div(a, b); }

// ---------------------------------------------------------------- bremsstrahlung
// q < qe_max decides whether the electron term exists (physics.hh:142):
// against a lean qe_max, and in IEEE arithmetic like the reference when q is
// within 64 ulp of it.
__device__ __forceinline__ bool brems_below(double E, double q, const noa_dcs_consts &c) {
    const double qe_lean = E * lean_rcp(1. + c.br_half_m2 * lean_rcp(ME * E));
    const long long dist = __double_as_longlong(q) - __double_as_longlong(qe_lean);
    if (dist < 64 && dist > -64)
        return brems_below_qe(E, q, c);
    return q < qe_lean;
}

__device__ __forceinline__ double brems_fp64(double K, double q, const noa_dcs_consts &c) {
    const double mass = c.mass;
    const double sqrte = 1.648721271;
    const double E = K + mass;
    const double invE = lean_rcp(E);
    const double delta_factor = c.br_half_m2 * invE;
    const bool below = brems_below(E, q, c);
    const double nu = __ddiv_rn(q, E);  // as the reference: 1 - nu cancels as q -> E
    const double delta = delta_factor * nu * lean_rcp(1. - nu);
    const double Phi_n = clamp0(lean_log(c.br_BZ_n * (mass + delta * c.br_Dn_sqrte_m2) *
                                         lean_rcp(c.br_D_n * (ME + delta * sqrte * c.br_BZ_n))));
    double Phi_e = 0.;
    if (below)
        Phi_e = clamp0(lean_log(c.br_BZe_mass *
                                lean_rcp((1. + delta * c.br_phie_factor) * (ME + delta * sqrte * c.br_BZ_e))));
    const double dcs = c.br_dcs_factor * (c.Zd * Phi_n + Phi_e) * (4. / 3. * (lean_rcp(nu) - 1.) + nu);
    return (dcs < 0.) ? 0. : dcs * c.scale_A;
}

// ---------------------------------------------------------------- pair production
// The rare part of pprod_live, out of line so that the kernels that inline
// pprod_live once per item keep one copy of it: the float-float argmin
// (~1e-13 relative here), whose distance from 1 decides beyond 1e-10, and
// the IEEE argmin near q = 4 me (1 - x0 < 1e-4, where 1 - x0 amplifies the
// error of x0), for extreme K, or within 1e-10.  Scalars only (a reference
// to the constants would copy them to local memory).
static __device__ __noinline__ bool pprod_live_tail(double K, double q, double mass, float inv_mass_h, float inv_mass_l,
                                             float x0) {
    noa_dcs_consts c;  // pprod_argmin_ff / _exact read only these three fields
    c.mass = mass;
    c.inv_mass_h = inv_mass_h;
    c.inv_mass_l = inv_mass_l;
    if (x0 < 0.9999f && fpconv::f32(K) < 1e15f) {
        const FF am = pprod_argmin_ff(K, q, c);
        const float d = (am.h - 1.f) + am.l;  // am.h - 1 is exact for am.h in [0.5, 2]
        if (am.h >= 0.5f && am.h <= 2.f && fabsf(d) > 1e-10f)
            return d < 0.f;
        if (am.h > 1e-30f && am.h < 0.5f)
            return true;
        if (am.h > 2.f && am.h < 1e30f)
            return false;
    }
    const double am = pprod_argmin_exact(K, q, c);
    return !((am >= 1.) || (am <= 0.));
}

// The whole open / closed decision in the reference's IEEE arithmetic
// (dcs.hh:151-156 and the argmin check), out of line: reached only where float
// cannot decide, so that the inlined fast path carries no FP64 comparison
// (the compiler would otherwise evaluate the short exact tests
// unconditionally, as predicated FP64 instructions, for every pair).
static __device__ __noinline__ bool pprod_live_exact(double K, double q, double mass, double shift,
                                                     float inv_mass_h, float inv_mass_l) {
    if (q <= 4. * ME)
        return false;
    if (q >= K + shift)
        return false;
    return pprod_live_tail(K, q, mass, inv_mass_h, inv_mass_l, 1.f);
}

__device__ __forceinline__ bool pprod_live(double K, double q, const noa_dcs_consts &c) {
    // NaN outside the normal float range: the range test below fails there
    const float Kf = fpconv::f32_normal(K), qf = fpconv::f32_normal(q);
    if (!(Kf > 1e-20f && Kf < 1e30f && qf > 1e-20f && qf < 1e30f))  // outside the float-safe range (and NaN)
        return pprod_live_exact(K, q, c.mass, c.pp_kmax_shift, c.inv_mass_h, c.inv_mass_l);
    // q <= 4 me and q >= K + m (1 - 0.75 sqrt(e) Z^1/3) (dcs.hh:151-156) in
    // float, with the IEEE comparison within a relative margin of 1e-5
    constexpr float four_me = (float)(4. * ME);
    if (qf < four_me * 0.99999f)
        return false;
    const float shift = c.pp_kmax_shift_f;
    const float ub = Kf + shift, margin = 1e-5f * (Kf + fabsf(shift));
    if (qf >= ub + margin)
        return false;
    if (!(qf > four_me * 1.00001f) || !(qf <= ub - margin))
        return pprod_live_exact(K, q, c.mass, c.pp_kmax_shift, c.inv_mass_h, c.inv_mass_l);
    // argmin in float, with K - q (gamma - q/m = 1 + (K - q)/m) as a
    // float-float difference; the reference's IEEE value decides only within
    // 1e-5 of a bound
    const FF kmq = ff_add(ff_split(K), ff_neg(ff_split(q)));
    const float im = c.inv_mass_h;
    const float x0 = four_me * lean64::rcp_approx(qf);
    const float gamma = 1.f + Kf * im;
    const float x1 = 6.f * lean64::rcp_approx(gamma * (1.f + (kmq.h + kmq.l) * im));
    const float a = (x0 + 2.f * (1.f - x0) * x1) * lean64::rcp_approx(1.f + (1.f - x1) * sqrtf(fmaxf(1.f - x0, 0.f)));
    if (fabsf(a - 1.f) > 1e-5f && a > 1e-30f && a < 1e30f && x0 < 0.9f)
        return a < 1.f;
    return pprod_live_tail(K, q, c.mass, c.inv_mass_h, c.inv_mass_l, x0);
}

__device__ __forceinline__ double pprod_fp64(double K, double q, const noa_dcs_consts &c) {
    if (q <= 4. * ME)
        return 0.;
    if (q >= K + c.pp_kmax_shift)
        return 0.;
    const double argmin = pprod_argmin_exact(K, q, c);
    if ((argmin >= 1.) || (argmin <= 0.))
        return 0.;
    const double mass = c.mass;
    const double E = K + mass;
    const double nu = __ddiv_rn(q, E);
    const double beta = 0.5 * nu * nu * ol_rcp(1. - nu);
    const double xi_factor = c.pp_half_r2 * beta;
    const double tmin = ol_log(argmin);
    // Le's two logs share one: log(AZ13 sqrt(xe) q / D1) - log(D2)/2 = log(AZ13^2 q^2 xe / (D1^2 D2)) / 2
    const double aq2 = (c.pp_AZ13 * q) * (c.pp_AZ13 * q);
    const double b2 = 2. * beta, b15 = 1.5 * beta, b3 = 3. * beta, b4 = 4. * beta;

    double I = 0.;
#pragma unroll 1  // rolled: 1% faster than unrolled on GB300 (smaller code, same FP64 work)
    for (int j = 0; j < 8; j++) {
        const double eps = ol_exp(kGL8X[j] * tmin);
        const double rho = 1. - eps;
        const double rho2 = rho * rho;
        const double rho21 = eps * (2. - eps);
        const double xi = xi_factor * rho21;
        const double xi_i = ol_rcp(xi);
        const double opxi = 1. + xi;
        const double inv_opxi = ol_rcp(opxi);

        double Be;
        if (bits_ge(xi, 1E+03))
            Be = 0.5 * xi_i * ((3. - rho2) + b2 * (1. + rho2));
        else
            Be = ((2. + rho2) * (1. + beta) + xi * (3. + rho2)) * ol_log(1. + xi_i) + (rho21 - beta) * inv_opxi -
                 3. - rho2;
        const double Ye = ol_div(5. - rho2 + b4 * (1. + rho2),
                                   2. * (1. + b3) * ol_log(3. + xi_i) - rho2 - b2 * (2. - rho2));
        const double xe = opxi * (1. + Ye);
        const double cLi = c.pp_cL * ol_rcp(rho21);
        const double d1 = q + cLi * xe;
        const double Le = 0.5 * ol_log(aq2 * xe * ol_rcp(d1 * d1 * (1. + c.pp_cLe * xe)));
        const double Phi_e = clamp0(Be * Le);

        double Bmu;
        if (!bits_ge(xi, 1.0000000000000002E-03))  // xi <= 1e-3
            Bmu = 0.5 * xi * (5. - rho2 + beta * (3. + rho2));
        else
            Bmu = ((1. + rho2) * (1. + b15) - xi_i * (1. + b2) * rho21) * ol_log(opxi) +
                  xi * (rho21 - beta) * inv_opxi + (1. + b2) * rho21;
        const double Ymu = ol_div(4. + rho2 + b3 * (1. + rho2),
                                    (1. + rho2) * (1.5 + b2) * ol_log(3. + xi) + 1. - 1.5 * rho2);
        const double xmu = opxi * (1. + Ymu);
        const double Lmu = ol_log(c.pp_r_AZ13 * q * ol_rcp(c.pp_15_Z13 * (q + cLi * xmu)));
        const double Phi_mu = clamp0(Bmu * Lmu);
        const double f = -(Phi_e + Phi_mu * c.pp_inv_r2) * (1. - rho) * tmin;
        I = fma(f, kGL8W[j], I);
    }

    const double gamma = __dadd_rn(1., __ddiv_rn(K, mass));
    double zeta = 0.;
    if (!(gamma <= 35.)) {
        zeta = 0.073 * ol_log(gamma * ol_rcp(1. + c.pp_gamma1 * gamma * c.pp_Z13 * c.pp_Z13)) - 0.26;
        if (zeta <= 0.)
            zeta = 0.;
        else
            zeta = ol_div(zeta, 0.058 * ol_log(gamma * ol_rcp(1. + c.pp_gamma2 * gamma * c.pp_Z13)) - 0.14);
    }
    const double dcs = ol_div(c.pp_cZ * (c.Zd + zeta) * (E - q) * I, q * E);
    return (dcs < 0.) ? 0. : dcs * (mass + K) * c.scale_A;
}

// ---------------------------------------------------------------- photonuclear
// photo_window's open / closed decision (dcs.hh:357-381), float first: in
// float every bound is decided with a relative margin of 1e-5 (1e-4 of the
// terms for Q2max >= Q2min, whose float difference cancels near q_min; with
// q_min = mpi (1 + mpi / 2M), Q2max = 2M (q - q_min) exactly in real
// arithmetic), far above float rounding; pairs within a margin, and inputs
// outside the float-safe range (zero, NaN, inf, huge), take the exact IEEE
// check.  Only the closed / open answer is taken from float, never a value.
__device__ __forceinline__ bool photo_live(double K, double q, const noa_dcs_consts &c) {
    // NaN outside the normal float range: the range test below fails there
    const float Kf = fpconv::f32_normal(K), qf = fpconv::f32_normal(q);
    if (Kf >= 1e-30f && Kf <= 1e30f && qf >= 1e-30f && qf <= 1e30f) {
        constexpr float lo = 0.99999f, hi = 1.00001f;
        const float qmin = c.ph_q_min_f, cut = 2E-03f * Kf;
        if (qf < lo || qf < cut * lo || qf > Kf * hi || qf < qmin * lo)
            return false;  // q < 1, q < 2e-3 K, q >= E - m (= K to an ulp), q <= q_min
        if (!(qf < hi || qf < cut * hi || qf > Kf * lo || qf < qmin * hi)) {
            const float m = c.mass_h;
            const float Ef = Kf + m, Emq = fpconv::f32_normal(K + c.mass - q);  // q < K (1 - 1e-5): no cancellation
            const float y = qf / Ef, omy = Emq / Ef;
            const float Q2min = m * m * y * y / omy;
            const float Q2max = (float)(2.0 * PH_M) * (qf - qmin);
            const float margin = 1e-4f * ((float)(2.0 * PH_M) * qf + Q2min);
            if (Q2max < Q2min - margin)
                return false;
            if (Q2max > Q2min + margin)
                return true;
        }
    }
    double a, b;
    return photo_window(K, q, c, a, b);
}

__device__ __forceinline__ double photo_fp64(double K, double q, const noa_dcs_consts &c) {
    double Q2min, Q2max;
    if (!photo_window(K, q, c, Q2min, Q2max))
        return 0.;
    const double mass = c.mass;
    const double E = K + mass;
    const double y = __ddiv_rn(q, E);
    const double pQ2min = ol_log(Q2min);
    const double pQ2max = ol_log(Q2max);
    const double dpQ2 = pQ2max - pQ2min;
    const double pQ2c = 0.5 * (pQ2max + pQ2min);

    // ALLM parameters, dcs.hh:262-288.
    const double m02 = 0.31985, mP2 = 49.457, mR2 = 0.15052, Q02 = 0.52544;
    const double cP1 = 0.28067, cP2 = 0.22291, cP3 = 2.1979;
    const double aP1 = -0.0808, aP2 = -0.44812, aP3 = 1.1709;
    const double bP1 = 0.36292, bP2 = 1.8917, bP3 = 1.8439;
    const double cR1 = 0.80107, cR2 = 0.97307, cR3 = 3.4942;
    const double aR1 = 0.58400, aR2 = 0.37888, aR3 = 2.6063;
    const double bR1 = 0.01147, bR2 = 3.7582, bR3 = 0.49338;
    const double M2 = 0.8803505929;
    const double inv_lambda2 = 1. / 0.06527;
    const double inv_ln10 = 0.43429448190325182765;

    const double cf = 2.603096E-35;
    const double invEE = ol_rcp(E * E);
    const double inv_q = ol_rcp(q);
    const double Mq = PH_M * q;
    const double inv_Mq = ol_rcp(Mq);
    const double two_Mq = 2. * Mq;
    const double two_m2 = 2 * mass * mass;
    const double yy = y * y;
    double ds = 0.;
#pragma unroll 1
    for (int j = 0; j < 9; j++) {
        const double Q2 = ol_exp(pQ2c + 0.5 * dpQ2 * kGL9X[j]);
        const double invQ2 = ol_rcp(Q2);
        const double x = 0.5 * Q2 * inv_Mq;
        // ALLM F2, dcs.hh:289-306
        const double W2 = M2 + Q2 * (two_Mq * invQ2 - 1.0);
        const double t = ol_log(ol_log((Q2 + Q02) * inv_lambda2) * c.ph_inv_log_q02);
        const double xP = (Q2 + mP2) * ol_rcp(Q2 + mP2 + W2 - M2);
        const double xR = (Q2 + mR2) * ol_rcp(Q2 + mR2 + W2 - M2);
        const double lnt = ol_log(t);
        const double cP = cP1 + (cP1 - cP2) * (ol_rcp(1.0 + ol_exp(cP3 * lnt)) - 1.0);
        const double aP = aP1 + (aP1 - aP2) * (ol_rcp(1.0 + ol_exp(aP3 * lnt)) - 1.0);
        const double bP = bP1 + bP2 * ol_exp(bP3 * lnt);
        const double cR = cR1 + cR2 * ol_exp(cR3 * lnt);
        const double aR = aR1 + aR2 * ol_exp(aR3 * lnt);
        const double bR = bR1 + bR2 * ol_exp(bR3 * lnt);
        const double l1x = ol_log(1 - x);
        const double F2P = cP * ol_exp(aP * ol_log(xP) + bP * l1x);
        const double F2R = cR * ol_exp(aR * ol_log(xR) + bR * l1x);
        const double F2p = Q2 * ol_rcp(Q2 + m02) * (F2P + F2R);
        // DRSS shadowing, dcs.hh:310-319
        double a = 1.0;
        if (x < 0.0014)
            a = c.ph_a_low;
        else if (x < 0.04)
            a = ol_exp((0.069 * (ol_log(x) * inv_ln10) + 0.097) * c.ph_logA);
        const double F2A = 0.5 * c.A * a * (2.0 + x * (-1.85 + x * (2.45 + x * (-2.35 + x)))) * F2p;
        // Whitlow R, dcs.hh:322-332
        const bool low = !bits_ge(Q2, 0.3);
        const double q2 = low ? 0.3 : Q2;
        const double inv_q2 = low ? 1. / 0.3 : invQ2;
        const double theta = 1 + 12.0 * q2 * 0.015625 * ol_rcp((1.0 + q2) * (0.015625 + x * x));
        const double R = 0.635 * theta * ol_rcp(ol_log(q2 * 25.)) + 0.5747 * inv_q2 -
                         0.3534 * ol_rcp(0.09 + q2 * q2);
        // dcs.hh:348-354
        const double dds = (1 - y + 0.5 * (1 - two_m2 * invQ2) * (yy + Q2 * invEE) * ol_rcp(1 + R)) *
                               (invQ2 * invQ2) -
                           0.25 * invEE * invQ2;
        const double d2 = cf * F2A * dds * inv_q;
        ds = fma(d2 * Q2, kGL9W[j], ds);
    }
    return (ds < 0.) ? 0. : 0.5 * ds * dpQ2 * (mass + K) * c.scale_A;
}

// Out-of-line entries of the two quadrature bodies for the FP32C redo paths
// (FP32C, batched FP32C and surrogate fallback kernels): the redo runs for
// 0-0.5% of the open pairs, and inlined it would set the register budget of
// the whole kernel.  Photonuclear's FP32C kernel runs 7% faster with it.
static __device__ __noinline__ double pprod_fp64_ol(double K, double q, const noa_dcs_consts &c) {
    return pprod_fp64(K, q, c);
}
static __device__ __noinline__ double photo_fp64_ol(double K, double q, const noa_dcs_consts &c) {
    return photo_fp64(K, q, c);
}

// ---------------------------------------------------------------- ionisation
// ionisation's first exit (dcs.hh:413-419: W_max < 5% K or q > W_max),
// decided in float first: W_max = 2 me K (K + 2 mass) / ((mass + me)^2 +
// 2 me K) has only positive terms, so its float value is within a few float
// ulps; each bound is decided with a relative margin of 1e-5.  1: the exit is
// not taken, 0: it is taken, -1: within a margin or outside the float-safe
// range (zero, NaN, inf, huge), where the caller takes the exact IEEE test.
// Only the decision is taken from float, never a value.
__device__ __forceinline__ int ion_first_exit(double K, double q, const noa_dcs_consts &c) {
    const float Kf = fpconv::f32_normal(K), qf = fpconv::f32_normal(q);  // NaN outside the normal range
    if (!(Kf >= 1e-30f && Kf <= 1e15f && qf >= 1e-30f && qf <= 1e30f))
        return -1;
    constexpr float me = (float)NOA_ELECTRON_MASS;
    const float W = 2.f * me * Kf * (Kf + 2.f * c.mass_h) / (c.io_cm_h + 2.f * me * Kf);
    constexpr float lo = 0.99999f, hi = 1.00001f;
    const float cut = (float)NOA_X_FRACTION * Kf;
    if (W < cut * lo || qf > W * hi)
        return 0;
    return (W > cut * hi && qf < W * lo) ? 1 : -1;
}

__device__ __forceinline__ double ion_fp64(double K, double q, const noa_dcs_consts &c) {
    const double mass = c.mass;
    const double P2 = K * (K + 2. * mass);
    const double E = K + mass;
    const int first = ion_first_exit(K, q, c);
    double inv_Wmax;
    if (first < 0) {
        const double Wmax = ion_wmax(P2, E, c);
        if ((Wmax < NOA_X_FRACTION * K) || (q > Wmax))
            return 0.;
        inv_Wmax = lean_rcp(Wmax);
    } else if (first == 0) {
        return 0.;
    } else {
        // 1 / W_max = (mass^2 + me (me + 2 E)) / (2 me P2), lean
        inv_Wmax = (mass * mass + ME * (ME + 2. * E)) * lean_rcp(2. * ME * P2);
    }
    if (q <= c.io_Wmin)
        return 0.;
    const double inv_P2 = lean_rcp(P2);
    const double inv_q = lean_rcp(q);
    const double a0 = 0.5 * inv_P2;
    const double a1 = -inv_Wmax;
    const double a2 = E * E * inv_P2;
    const double cs = c.io_cZA * E * (a0 + inv_q * (a1 + a2 * inv_q));
    double Delta = 0.;
    if (K >= c.io_k_rad) {
        const double L1 = lean_log(1. + q * (2. / ME));
        Delta = 1.16141E-03 * L1 * (lean_log(4. * E * (E - q) * c.inv_m2) - L1);
    }
    return cs * (1. + Delta);
}

} // namespace noa_dcs
