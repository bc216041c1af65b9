/*
 * FP32-compensated ("FP32C") forms of the four muon DCS processes.
 *
 * The quadrature bodies run in FP32, with compensated node sums.  Where
 * float would lose the answer the arithmetic is float-float (FF, ~2^-44 on
 * the FP32 pipe) or FP64: the kinematic bounds are decided in float with a
 * margin and exactly (FP64 / FF) inside it, so the zero pattern is the
 * reference's; the kinematic-edge differences E - q (FP64), 1 - nu and
 * 2Mq - Q2; the node arguments t tmin and log Q2 as float pairs; the
 * kinematic-limit logs log(argmin), log Q2min and log(Q2max / Q2min) in FF;
 * and the final macroscopic scaling in double (its constants are far below
 * FLT_MIN).
 *
 * Reformulations that remove float cancellations, all exact algebra:
 *  - pair production Be / Bmu, dcs.hh:188-216: the terms
 *    xi log(1 + 1/xi) - 1 and log(1 + xi)/xi - 1 cancel to O(1/xi) (O(xi)); they
 *    are evaluated as u H(u) with H(u) = (log1p(u) - u)/u^2 from a fitted
 *    polynomial (gen_fp32c_poly.py) for u <= 1;
 *  - pair production Le, dcs.hh:201-202: one log of (AZ13 q/D1)^2 xe/D2;
 *  - rho = 1 - exp(t tmin) as -expm1, and (1 - rho) as exp(t tmin);
 *  - photonuclear ALLM, dcs.hh:289-292: W2 - M2 = Q2 (1/x - 1) = 2Mq - Q2, so
 *    xP = (Q2 + mP2)/(mP2 + 2Mq); t = log(1 + log1p(Q2/Q02)/log(Q02/L2));
 *    1 - x = (2Mq - Q2)/(2Mq) with 2Mq - Q2 = (2Mq - Q2max) - Q2max expm1(.);
 *  - cP, aP: 1/(1 + e) - 1 = -e/(1 + e).
 *
 * Each evaluation also returns `est`, a running estimate of its relative
 * float rounding error (a few units of 2^-24 per operation, scaled by the size
 * of what cancels), or infinity where a branch or clamp of the reference sits
 * within rounding distance.  When est exceeds the caller's tolerance the
 * kernel evaluates that pair in FP64 instead (pair production: first again
 * in FP32 with its screening log in FF, pprod_fp32c<false, true>).
 *
 * Written for host and device (NOA_HD) so that the same source can be
 * checked against the CPU oracle.
 */
#pragma once

#include "dcs_common.cuh"

namespace noa_dcs {

constexpr float U32 = 5.9604645e-08f; // 2^-24

// The node loops stay rolled (unroll factor 1 unless NOA_FP32C_NODE_UNROLL
// sets another): fully unrolled, the long FP32 bodies overflowed the
// instruction cache (ncu "no instruction" stalls), and rolled they run 16%
// (pair production) and 13% (photonuclear) faster on GB300.
#define NOA_STRINGIFY(x) #x
#define NOA_PRAGMA(x) _Pragma(NOA_STRINGIFY(x))
#ifndef NOA_FP32C_NODE_UNROLL
#define NOA_FP32C_NODE_UNROLL 1
#endif
#define NOA_UNROLL_NODES NOA_PRAGMA(unroll NOA_FP32C_NODE_UNROLL)

// Gauss-Legendre literals of numerics.hh:116-121 (8 nodes on [0, 1]) and
// :137-144 (9 nodes on [-1, 1]), each node split into floats hi + lo that sum
// to the double literal to 2^-48; weights rounded to float.  Constant memory
// on the device (every lane of a warp reads the same node).
#if defined(__CUDA_ARCH__)
#define NOA_F32_TABLE static __constant__ const
#else
#define NOA_F32_TABLE static const
#endif
NOA_F32_TABLE float kF8XH[8] = {1.985507086e-02f, 1.016667634e-01f, 2.372338027e-01f, 4.082826674e-01f,
                                5.917173028e-01f, 7.627661824e-01f, 8.983332515e-01f, 9.801449180e-01f};
NOA_F32_TABLE float kF8XL[8] = {-8.591938272e-10f, -3.424873274e-09f, -2.676200817e-09f, 1.260154736e-08f,
                                1.720077591e-08f,  1.757736179e-08f,  -1.147628748e-08f, 1.203506450e-08f};
NOA_F32_TABLE float kF8W[8] = {0.05061427f, 0.11119052f, 0.15685332f, 0.18134189f,
                               0.18134189f, 0.15685332f, 0.11119052f, 0.05061427f};
NOA_F32_TABLE float kF9XH[9] = {0.000000000e+00f, -8.360310793e-01f, 8.360310793e-01f, -9.681602120e-01f,
                                9.681602120e-01f, -3.242534101e-01f, 3.242534101e-01f, -6.133714318e-01f,
                                6.133714318e-01f};
NOA_F32_TABLE float kF9XL[9] = {0.000000000e+00f, -2.803433929e-08f, 2.803433929e-08f, -2.746767791e-08f,
                                2.746767791e-08f, -1.330287169e-08f, 1.330287169e-08f, -8.730451917e-10f,
                                8.730451917e-10f};
NOA_F32_TABLE float kF9W[9] = {0.3302393550012598f, 0.1806481606948574f, 0.1806481606948574f,
                               0.0812743883615744f, 0.0812743883615744f, 0.3123470770400029f,
                               0.3123470770400029f, 0.2606106964029354f, 0.2606106964029354f};

NOA_HD float f_rcp(float x) {
#if defined(__CUDA_ARCH__)
    const float y = lean64::rcp_approx(x);
    // one Newton step; 1/0, 1/inf and NaN keep the approximation's IEEE value
    return (fabsf(y) < INFINITY && y != 0.f) ? fmaf(y, fmaf(-x, y, 1.f), y) : y;
#else
    return 1.f / x;
#endif
}
NOA_HD float f_div(float a, float b) { return a * f_rcp(b); }
NOA_HD float f_clamp0(float v) { return v < 0.f ? 0.f : v; }

// H(u) = (log1p(u) - u) / u^2 on [0, 1] (gen_fp32c_poly.py, 9.7e-9 truncation).
NOA_HD float poly_H(float u) {
    float h = 2.873883747e-03f;
    h = fmaf(h, u, -1.751224284e-02f);
    h = fmaf(h, u, 4.993118107e-02f);
    h = fmaf(h, u, -9.202963259e-02f);
    h = fmaf(h, u, 1.307132827e-01f);
    h = fmaf(h, u, -1.637850887e-01f);
    h = fmaf(h, u, 1.995935617e-01f);
    h = fmaf(h, u, -2.499702413e-01f);
    h = fmaf(h, u, 3.333324756e-01f);
    return fmaf(h, u, -4.999999959e-01f);
}

// Compensated float accumulator (Neumaier's variant of Kahan summation).
struct KSum {
    float s = 0.f, c = 0.f;
    NOA_HD void add(float v) {
        const float t = s + v;
        c += (fabsf(s) >= fabsf(v)) ? ((s - t) + v) : ((v - t) + s);
        s = t;
    }
    NOA_HD double value() const { return fpconv::f64(s) + fpconv::f64(c); }
};

// exp(uh + ul) and -expm1(uh + ul) for a double argument split into floats.
NOA_HD void f_exp_split(double u, float &e, float &em1) {
    const float uh = fpconv::f32(u);
    const float ul = fpconv::f32(u - fpconv::f64(uh));
    const float eh = expf(uh);
    e = fmaf(eh, ul, eh);
    em1 = fmaf(eh, ul, expm1f(uh));
}

// The same for u = x t with x = xh + xl and t = th + tl float-float pairs,
// entirely in FP32: x t is formed as a float-float product (the FMA gives
// xh th exactly), so exp sees u to ~2^-48 without an FP64 instruction.
NOA_HD void f_exp_split_ff(float xh, float xl, float th, float tl, float &e, float &em1) {
    const float ph = xh * th;
    const float pl = fmaf(xh, th, -ph) + (xh * tl + xl * th);
    const float uh = ph + pl;
    const float ul = pl - (uh - ph);
    const float eh = expf(uh);
    e = fmaf(eh, ul, eh);
    em1 = fmaf(eh, ul, expm1f(uh));
}

// exp(c + h x) and expm1 of it, with c = ch + cl, h = hh + hl and
// x = xh + xl float-float pairs, entirely in FP32 (as f_exp_split_ff).
NOA_HD void f_exp_split_aff(float ch, float cl, float hh, float hl, float xh, float xl, float &e, float &em1) {
    const float ph = hh * xh;
    const float pl = fmaf(hh, xh, -ph) + (hh * xl + hl * xh);
    // (ch + ph) as a float-float sum, then the low parts
    const float s = ch + ph;
    const float bb = s - ch;
    const float sl = (ch - (s - bb)) + (ph - bb) + (cl + pl);
    const float uh = s + sl;
    const float ul = sl - (uh - s);
    const float eh = expf(uh);
    e = fmaf(eh, ul, eh);
    em1 = fmaf(eh, ul, expm1f(uh));
}

// ---------------------------------------------------------------- float-float exp / log
// 2^(j/64), j = 0..63, as float pairs hi + lo (to ~2^-48), for ff_exp.
NOA_F32_TABLE float kExp64H[64] = {
    1.000000000e+00f, 1.010889292e+00f, 1.021897197e+00f, 1.033024907e+00f, 1.044273734e+00f, 1.055645227e+00f,
    1.067140460e+00f, 1.078760743e+00f, 1.090507746e+00f, 1.102382541e+00f, 1.114386797e+00f, 1.126521587e+00f,
    1.138788581e+00f, 1.151189208e+00f, 1.163724899e+00f, 1.176396966e+00f, 1.189207077e+00f, 1.202156782e+00f,
    1.215247393e+00f, 1.228480577e+00f, 1.241857767e+00f, 1.255380750e+00f, 1.269050956e+00f, 1.282870054e+00f,
    1.296839595e+00f, 1.310961246e+00f, 1.325236678e+00f, 1.339667559e+00f, 1.354255557e+00f, 1.369002461e+00f,
    1.383909941e+00f, 1.398979664e+00f, 1.414213538e+00f, 1.429613352e+00f, 1.445180774e+00f, 1.460917830e+00f,
    1.476826191e+00f, 1.492907763e+00f, 1.509164453e+00f, 1.525598168e+00f, 1.542210817e+00f, 1.559004426e+00f,
    1.575980902e+00f, 1.593142152e+00f, 1.610490322e+00f, 1.628027439e+00f, 1.645755529e+00f, 1.663676620e+00f,
    1.681792855e+00f, 1.700106382e+00f, 1.718619347e+00f, 1.737333894e+00f, 1.756252170e+00f, 1.775376439e+00f,
    1.794709086e+00f, 1.814252138e+00f, 1.834008098e+00f, 1.853979111e+00f, 1.874167681e+00f, 1.894575953e+00f,
    1.915206552e+00f, 1.936061740e+00f, 1.957144141e+00f, 1.978456020e+00f};
NOA_F32_TABLE float kExp64L[64] = {
    0.000000000e+00f, -5.711605411e-09f, -4.811559862e-08f, -2.809089317e-08f, 4.833470157e-08f,
    -4.907169426e-08f, -5.933751979e-08f, 5.461594554e-08f, -1.307753994e-08f, 4.260501996e-08f,
    -5.435540018e-08f, 3.123641434e-08f, 5.386222313e-08f, 2.192228266e-08f, -4.051441493e-08f,
    2.566975077e-08f, 3.797635273e-08f, -5.069756526e-08f, -3.267394888e-08f, -4.136200360e-08f,
    4.496838102e-08f, 7.322237483e-09f, 1.419333318e-09f, -3.816621685e-08f, -4.018999533e-08f,
    -3.496571566e-08f, -3.496373324e-08f, -3.461673970e-08f, -1.012334927e-08f, -3.845881835e-08f,
    -5.875577358e-08f, 8.689434061e-09f, 2.420323497e-08f, -1.342992917e-08f, 3.324199938e-08f,
    -3.628657552e-08f, -4.500898854e-08f, -3.423620143e-08f, -2.495937323e-08f, -1.762856883e-08f,
    8.070904833e-09f, -2.576466507e-08f, -5.661025426e-08f, -4.903136785e-10f, 9.836217174e-09f,
    -1.726008314e-08f, -5.124972091e-08f, -3.920298752e-08f, -2.475532668e-08f, -2.865147231e-08f,
    -4.849617596e-08f, -5.850223417e-08f, -9.235770371e-09f, 5.343197884e-08f, -1.141504491e-08f,
    3.736258236e-08f, -1.123927795e-08f, 1.436561181e-08f, -4.663005626e-08f, 2.810338451e-08f,
    9.845328108e-09f, 5.357072297e-08f, -1.702180441e-08f, 6.032726318e-09f};

// 2^n as a float, -126 <= n <= 127.
NOA_HD float f_pow2i(int n) {
#if defined(__CUDA_ARCH__)
    return __int_as_float((n + 127) << 23);
#else
    return ldexpf(1.f, n);
#endif
}

// exp(a) of a float-float a, -87 < a < 88, to ~2^-44 relative on the FP32
// pipe (Tang's table method): a = k ln2/64 + r with ln2/64 in three parts
// (Cody-Waite; k L1 is exact for |k| < 2^13), exp(r) - 1 = r + r^2/2 + r^3/6
// + r^4/24 + r^5/120 (|r| <= 0.0055, r^2 in float-float, the cubic tail in
// float), times 2^(j/64) from the table (j = k mod 64) and 2^(k div 64).
NOA_HD FF ff_exp(FF a) {
    const float kf = rintf(a.h * 92.33248262f);  // 64 / ln 2
    const int k = (int)kf;
    const float r1 = fmaf(-kf, 0.010833740234375f, a.h);  // exact
    const float ph = kf * -3.315538152e-06f;
    const float pl = fmaf(kf, -3.315538152e-06f, -ph);
    const FF r = ff_add(FF{r1, fmaf(-kf, 2.572804640e-14f, a.l)}, FF{-ph, -pl});
    const float rh = r.h;
    const float tail = rh * rh * rh * fmaf(rh, fmaf(rh, 1.f / 120.f, 1.f / 24.f), 1.f / 6.f);
    const FF r2 = ff_mul(r, r);
    const FF em1 = ff_add(r, ff_add(FF{0.5f * r2.h, 0.5f * r2.l}, FF{tail, 0.f}));
    const FF T{kExp64H[k & 63], kExp64L[k & 63]};
    const FF e = ff_add(T, ff_mul(T, em1));
    const float sc = f_pow2i(k >> 6);
    return FF{e.h * sc, e.l * sc};
}

// log(x) of a positive normal float-float x to ~2^-44 relative: the float
// log, corrected by t = x exp(-y0) - 1 (log(1 + t) = t - t^2/2, |t| ~ 1e-7).
NOA_HD FF ff_log(FF x) {
    const float y0 = logf(x.h);
    const FF t = ff_add(ff_mul(x, ff_exp(FF{-y0, 0.f})), FF{-1.f, 0.f});
    return ff_add(FF{y0, 0.f}, ff_add(t, FF{-0.5f * t.h * t.h, 0.f}));
}

// ---------------------------------------------------------------- bremsstrahlung
NOA_HD double brems_fp32c(double K, double q, const noa_dcs_consts &c, float &est) {
    est = 0.f;
    const float Kf = fpconv::f32(K), qf = fpconv::f32(q);
    if (!(Kf > 1e-20f && Kf < 1e30f && qf > 1e-20f && qf < 1e30f)) {  // NaN, q <= 0, extreme ranges: FP64
        est = INFINITY;
        return 0.;
    }
    // E = K + m and E - q in float-float; q within 1e-4 of E (or above it),
    // where that difference would lose digits, goes to FP64
    const FF EF = ff_add(ff_split(K), FF{c.mass_h, c.mass_l});
    const FF EmqF = ff_add(EF, ff_neg(ff_split(q)));
    const float Ef = EF.h, Emq = EmqF.h + EmqF.l;
    if (!(Emq > 1e-4f * Ef)) {
        est = INFINITY;
        return 0.;
    }
    // q < qe_max (physics.hh:142): float decision, exact when close
    const float qe = f_div(Ef, 1.f + fpconv::f32(c.br_half_m2) * f_rcp((float)ME * Ef));
    bool below = qf < qe;
    if (fabsf(qf - qe) <= 1e-5f * qe)
        below = brems_below_qe(K + c.mass, q, c);
    const float sqrte = 1.648721271f;
    // delta = 0.5 m^2 nu / (E (1 - nu)) = 0.5 m^2 q / (E (E - q))
    const float delta = fpconv::f32(c.br_half_m2) * qf * f_rcp(Ef * Emq);
    const float BZn = fpconv::f32(c.br_BZ_n), Dn = fpconv::f32(c.br_D_n), BZe = fpconv::f32(c.br_BZ_e);
    const float Phi_n = logf((BZn * (fpconv::f32(c.mass) + delta * fpconv::f32(c.br_Dn_sqrte_m2))) *
                             f_rcp(Dn * ((float)ME + delta * sqrte * BZn)));
    float Phi_e = 0.f;
    if (below)
        Phi_e = logf(fpconv::f32(c.br_BZe_mass) *
                     f_rcp((1.f + delta * fpconv::f32(c.br_phie_factor)) * ((float)ME + delta * sqrte * BZe)));
    const float Zf = fpconv::f32(c.Zd);
    const float S = Zf * f_clamp0(Phi_n) + f_clamp0(Phi_e);
    // 4/3 (1/nu - 1) + nu = 4/3 (E - q)/q + q/E
    const float fac = 1.33333333f * Emq * f_rcp(qf) + qf * f_rcp(Ef);
    const float err = Zf * 3.f * U32 + 3.f * U32 + 3.f * U32 * S;
    est = 2.0f * err * f_rcp(S);  // calibrated against the oracle: max error <= est
    if (!(S > 0.f) || !(Phi_n > 16.f * U32 || Phi_n < -16.f * U32) ||
        (below && !(Phi_e > 16.f * U32 || Phi_e < -16.f * U32)))
        est = INFINITY;
    const float sf = S * fac;
    return (sf < 0.f) ? 0. : fpconv::f64(sf) * c.br_scale;  // br_scale > 0: the sign is sf's
}

// ---------------------------------------------------------------- pair production
// CHECKED = false: the caller has already established with the exact bounds
// that the pair is open, and argmin is then formed in lean arithmetic (its
// relative error only matters for |tmin| < 1e-6, which is sent to FP64).
//
// FINE = true: the screening log Le and what it is built from (eps, xi, Ye,
// xe, the log arguments) in float-float arithmetic, the rest as in the float
// form.  Le is small (0.05-0.5) where Be Le carries the node, and its float
// absolute error of a few 2^-24 (from Ye's log and the chain before it) is
// what sends ~4% of the open pairs past a 1e-6 estimate; with Le to ~1e-13
// relative about one in a hundred of those stays above it.  About twice the
// FP32 work of the float form, for the pairs the float form rejects.
template <bool CHECKED = true, bool FINE = false>
NOA_HD double pprod_fp32c(double K, double q, const noa_dcs_consts &c, float &est) {
    est = 0.f;
    FF argmin;
    if (CHECKED) {
        if (q <= 4. * ME)
            return 0.;
        if (q >= K + c.pp_kmax_shift)
            return 0.;
        const double a = pprod_argmin_exact(K, q, c);
        if ((a >= 1.) || (a <= 0.))
            return 0.;
        argmin = ff_from(a);
    } else {
        argmin = pprod_argmin_ff(K, q, c);
    }
    const double mass = c.mass;
    const double E = K + mass;
    const double Emq = E - q;
    // beta = 0.5 nu^2 / (1 - nu) = 0.5 q^2 / (E (E - q))
    const double beta_d = 0.5 * q * q * d_rcp(E * Emq);
    // tmin = log(argmin) = tmin + tmin_lo, float-float log (~2^-44, no FP64)
    const FF tminF0 = ff_log(argmin);
    const float tmin = tminF0.h, tmin_lo = tminF0.l;
    const float beta = fpconv::f32(beta_d);
    const float xi_factor = fpconv::f32(c.pp_half_r2 * beta_d);
    const float qf = fpconv::f32(q);
    const float AZ13 = fpconv::f32(c.pp_AZ13), cL = fpconv::f32(c.pp_cL), cLe = fpconv::f32(c.pp_cLe);
    const float rAZ13 = fpconv::f32(c.pp_r_AZ13), Z13_15 = fpconv::f32(c.pp_15_Z13), inv_r2 = fpconv::f32(c.pp_inv_r2);
    const float b2 = 2.f * beta, b15 = 1.5f * beta, b3 = 3.f * beta, b4 = 4.f * beta;

    // float-float inputs of the screening log (FINE only)
    FF tminF{}, betaF{}, xfF{}, qF{}, cLF{}, cLeF{}, aq2F{};
    if (FINE) {
        tminF = tminF0;
        betaF = ff_from(beta_d);
        xfF = ff_from(c.pp_half_r2 * beta_d);
        qF = ff_from(q);
        cLF = ff_from(c.pp_cL);
        cLeF = ff_from(c.pp_cLe);
        aq2F = ff_mul(ff_from(c.pp_AZ13 * c.pp_AZ13), ff_mul(qF, qF));
    }

    KSum I;
    float err = 0.f;
    bool edge = !(fabsf(tmin) > 1e-6f);
    NOA_UNROLL_NODES
    for (int j = 0; j < 8; j++) {
        float eps, rho;
        f_exp_split_ff(kF8XH[j], kF8XL[j], tmin, tmin_lo, eps, rho);
        rho = -rho;
        const float rho2 = rho * rho;
        const float rho21 = eps * (2.f - eps);
        const float xi = xi_factor * rho21;
        const float xi_i = f_rcp(xi);
        const float opxi = 1.f + xi;
        const float inv_opxi = f_rcp(opxi);
        // branch thresholds of the reference (1e3, 1e-3) must be taken as it takes them
        edge |= fabsf(xi - 1e3f) <= 2e-4f || fabsf(xi - 1e-3f) <= 2e-10f;

        float Be, eBe;
        if (xi >= 1E+03f) {
            Be = 0.5f * xi_i * ((3.f - rho2) + b2 * (1.f + rho2));
            eBe = 2.f * U32 * Be;
        } else {
            const float A = (2.f + rho2) * (1.f + beta);
            float L, G;
            if (xi >= 1.f) {
                G = xi_i * poly_H(xi_i);  // xi log(1 + 1/xi) - 1
                L = xi_i * (1.f + G);     // log(1 + 1/xi)
            } else {
                L = log1pf(xi_i);
                G = xi * L - 1.f;
            }
            const float t1 = A * L, t2 = (3.f + rho2) * G, t3 = (rho21 - beta) * inv_opxi;
            Be = t1 + t2 + t3;
            eBe = 2.f * U32 * (fabsf(t1) + fabsf(t2) + fabsf(t3) + fabsf(beta) * inv_opxi);
        }
        const float Ye = f_div(5.f - rho2 + b4 * (1.f + rho2), 2.f * (1.f + b3) * logf(3.f + xi_i) - rho2 -
                                                                  b2 * (2.f - rho2));
        const float xe = opxi * (1.f + Ye);
        const float cLi = cL * f_rcp(rho21);
        float Le;
        if (FINE) {
            // Le = log(AZ13 q sqrt(xe) / D1) - log(D2) / 2 (dcs.hh:199-202) as one
            // float-float log of AZ13^2 q^2 xe / (D1^2 D2)
            const FF epsF = ff_exp(ff_mul(FF{kF8XH[j], kF8XL[j]}, tminF));
            const FF rhoF = ff_add(1.f, ff_neg(epsF));
            const FF rho2F = ff_mul(rhoF, rhoF);
            const FF r21F = ff_mul(epsF, ff_add(2.f, ff_neg(epsF)));
            const FF xiF = ff_mul(xfF, r21F);
            const FF L3 = ff_log(ff_add(3.f, ff_div(FF{1.f, 0.f}, xiF)));
            const FF num = ff_add(ff_add(5.f, ff_neg(rho2F)), ff_mul(ff_mul(4.f, betaF), ff_add(1.f, rho2F)));
            const FF den = ff_add(ff_add(ff_mul(ff_mul(2.f, ff_add(1.f, ff_mul(3.f, betaF))), L3), ff_neg(rho2F)),
                                  ff_neg(ff_mul(ff_mul(2.f, betaF), ff_add(2.f, ff_neg(rho2F)))));
            const FF xeF = ff_mul(ff_add(1.f, xiF), ff_add(1.f, ff_div(num, den)));
            const FF d1 = ff_add(qF, ff_mul(ff_div(cLF, r21F), xeF));
            const FF lg = ff_log(ff_div(ff_mul(aq2F, xeF), ff_mul(ff_mul(d1, d1), ff_add(1.f, ff_mul(cLeF, xeF)))));
            Le = 0.5f * (lg.h + lg.l);
        } else {
            const float r1 = AZ13 * qf * f_rcp(qf + cLi * xe);
            const float r2 = xe * f_rcp(1.f + cLe * xe);
            Le = 0.5f * logf(r1 * r1 * r2);
        }
        const float Phi_e = f_clamp0(Be * Le);

        float Bmu, eBmu;
        if (xi <= 1E-03f) {
            Bmu = 0.5f * xi * (5.f - rho2 + beta * (3.f + rho2));
            eBmu = 2.f * U32 * Bmu;
        } else {
            float L1, G2;
            if (xi <= 1.f) {
                G2 = xi * poly_H(xi);  // log(1 + xi)/xi - 1
                L1 = xi * (1.f + G2);  // log(1 + xi)
            } else {
                L1 = log1pf(xi);
                G2 = L1 * xi_i - 1.f;
            }
            const float s1 = (1.f + rho2) * (1.f + b15) * L1, s2 = (1.f + b2) * rho21 * G2,
                        s3 = xi * (rho21 - beta) * inv_opxi;
            Bmu = s1 - s2 + s3;
            eBmu = 2.f * U32 * (fabsf(s1) + fabsf(s2) + fabsf(s3) + xi * fabsf(beta) * inv_opxi);
        }
        const float Ymu = f_div(4.f + rho2 + b3 * (1.f + rho2),
                                (1.f + rho2) * (1.5f + b2) * logf(3.f + xi) + 1.f - 1.5f * rho2);
        const float xmu = opxi * (1.f + Ymu);
        const float Lmu = logf(rAZ13 * qf * f_rcp(Z13_15 * (qf + cLi * xmu)));
        const float Phi_mu = f_clamp0(Bmu * Lmu);
        const float g = -(Phi_e + Phi_mu * inv_r2) * eps * tmin;
        I.add(g * kF8W[j]);
        // error of this node: the logs to a few u absolute (Le 3 u, or 0.5 u
        // relative when FINE; Lmu 4 u: its argument carries the float error of
        // xmu), the B terms as tracked, the rest ~3 u relative
        const float eg = fabsf(eps * tmin) *
                         ((Phi_e > 0.f ? fabsf(Be) * (FINE ? fabsf(Le) : 3.f) * U32 + fabsf(Le) * eBe : 0.f) +
                          (Phi_mu > 0.f ? (fabsf(Bmu) * 4.f * U32 + fabsf(Lmu) * eBmu) * inv_r2 : 0.f)) +
                         fabsf(g) * 3.f * U32;
        err += eg * kF8W[j];
        // a screening log near zero decides the clamp; let FP64 decide it
        edge |= (fabsf(Le) < 64.f * U32) || (fabsf(Lmu) < 64.f * U32);
    }

    const double gamma = 1. + K * c.inv_mass;
    // zeta (dcs.hh:230-251) in float, with a bound on its float error; where
    // the cancellations in its numerator or denominator make that bound
    // matter (above 1e-7 of Z + zeta, e.g. for hydrogen), it is recomputed in
    // FP64 as in the plain kernel
    float zeta = 0.f, zeta_err = 0.f;
    if (!(gamma <= 35.)) {
        const float gf = fpconv::f32(gamma), Z13 = fpconv::f32(c.pp_Z13);
        const float L1 = logf(gf * f_rcp(1.f + fpconv::f32(c.pp_gamma1) * gf * Z13 * Z13));
        zeta = 0.073f * L1 - 0.26f;
        if (zeta <= 0.f) {
            zeta = 0.f;
        } else {
            const float L2 = logf(gf * f_rcp(1.f + fpconv::f32(c.pp_gamma2) * gf * Z13));
            const float den = 0.058f * L2 - 0.14f;
            const float ez = ((0.073f * (fabsf(L1) + 3.f) + 0.26f) * f_rcp(zeta) +
                              (0.058f * (fabsf(L2) + 3.f) + 0.14f) * f_rcp(fabsf(den)) + 2.f) * U32;
            zeta = f_div(zeta, den);
            zeta_err = fabsf(zeta) * ez;
            if (!(zeta_err <= 1e-7f * (fpconv::f32(c.Zd) + zeta))) {
                double zd = 0.073 * d_log(gamma * d_rcp(1. + c.pp_gamma1 * gamma * c.pp_Z13 * c.pp_Z13)) - 0.26;
                zd = zd <= 0. ? 0. : zd * d_rcp(0.058 * d_log(gamma * d_rcp(1. + c.pp_gamma2 * gamma * c.pp_Z13)) - 0.14);
                zeta = fpconv::f32(zd);
                zeta_err = fabsf(zeta) * U32;
            }
        }
        edge |= fabsf(gf - 35.f) < 1e-4f;
    }
    const double Id = I.value();
    // calibrated against the oracle on 2.4e8 host evaluations (10 elements, six
    // ranges of 4e6 seeded pairs, both forms): no pair above 1e-6 has an
    // estimate below 1.2e-6 (the estimate bounds the error with 17% to spare
    // at the tolerance); largest accepted error 7.5e-7
    est = edge ? INFINITY : 1.2f * err * f_rcp(fpconv::f32(fabs(Id))) + zeta_err * f_rcp(fpconv::f32(c.Zd) + zeta);
    const double dcs = c.pp_cZ * (c.Zd + fpconv::f64(zeta)) * Emq * Id * d_rcp(q * E);
    return (dcs < 0.) ? 0. : dcs * (mass + K) * c.scale_A;
}

// ---------------------------------------------------------------- photonuclear
// Float-pair constants of the photonuclear window: 2M, mpi, mpi^2, the ALLM
// masses mP2 and mR2 (dcs.hh:262-288, 370-381), and 2M mpi + mpi^2.
constexpr float kTwoMH = (float)(2. * PH_M), kTwoML = (float)(2. * PH_M - (double)kTwoMH);
constexpr float kMpiH = (float)PH_MPI, kMpiL = (float)(PH_MPI - (double)kMpiH);
constexpr float kMpi2H = (float)(PH_MPI * PH_MPI), kMpi2L = (float)(PH_MPI * PH_MPI - (double)kMpi2H);
constexpr float kMP2H = (float)49.457, kMP2L = (float)(49.457 - (double)kMP2H);
constexpr float kMR2H = (float)0.15052, kMR2L = (float)(0.15052 - (double)kMR2H);
constexpr float kDConst = (float)(2. * PH_M * PH_MPI + PH_MPI * PH_MPI);

// CHECKED = false: the caller has established that the pair is inside the
// kinematic window; Q2min / Q2max are then formed in lean arithmetic.
template <bool CHECKED = true>
NOA_HD double photo_fp32c(double K, double q, const noa_dcs_consts &c, float &est) {
    est = 0.f;
    const double mass = c.mass;
    // The window and its logs in float-float (~2^-44; FP64 only for E - q,
    // whose q -> E edge float-float of E and q would not resolve).  Q2min =
    // m^2 y^2 / (1 - y) = m^2 q^2 / (E (E - q)), Q2max = 2M (q - mpi) - mpi^2
    // (dcs.hh:377-381); log Q2max - log Q2min as one log of their ratio.
    FF Q2minF, Q2maxF;
    const double Emq_d = (K + mass) - q;
    const FF massF{c.mass_h, c.mass_l};
    FF KF, qF;
    if (CHECKED) {
        double a, b;
        if (!photo_window(K, q, c, a, b))
            return 0.;
        Q2minF = ff_from(a);
        Q2maxF = ff_from(b);
        KF = ff_from(K);
        qF = ff_from(q);
    } else {
        // the caller established the window (1 <= q < K); float-float holds
        // q^2 and the window for K below 1e15, FP64 takes the rest
        if (!(fpconv::f32(K) < 1e15f)) {
            est = INFINITY;
            return 0.;
        }
        KF = ff_split(K);
        qF = ff_split(q);
    }
    const FF EF = ff_add(KF, massF);
    const FF EmqF = ff_from(Emq_d);
    if (!CHECKED) {
        Q2minF = ff_div(ff_mul(ff_mul(massF, massF), ff_mul(qF, qF)), ff_mul(EF, EmqF));
        Q2maxF = ff_add(ff_mul(FF{kTwoMH, kTwoML}, ff_add(qF, FF{-kMpiH, -kMpiL})), FF{-kMpi2H, -kMpi2L});
    }
    const FF dpQ2F = ff_log(ff_div(Q2maxF, Q2minF));
    const FF pQ2cF = ff_add(ff_log(Q2minF), FF{0.5f * dpQ2F.h, 0.5f * dpQ2F.l});
    const FF inv_EF = ff_div(FF{1.f, 0.f}, EF);
    const float omy = ff_mul(EmqF, inv_EF).h;  // 1 - y, kinematic edge q -> E
    const float y = ff_mul(qF, inv_EF).h;
    const FF two_MqF = ff_mul(FF{kTwoMH, kTwoML}, qF);
    const float D = kDConst;  // 2Mq - Q2max = 2 M mpi + mpi^2
    const float inv_2Mq = ff_div(FF{1.f, 0.f}, two_MqF).h;
    const float inv_Mq = 2.f * inv_2Mq;
    const float Q2maxf = Q2maxF.h;
    const float half_dp = 0.5f * dpQ2F.h;
    // node abscissae log Q2 = pQ2c + (dpQ2 / 2) x_j in float-float
    const float pc_h = pQ2cF.h, pc_l = pQ2cF.l;
    const float hd_h = half_dp, hd_l = 0.5f * dpQ2F.l;

    const float m02 = 0.31985f, mP2 = 49.457f, mR2 = 0.15052f;
    const float cP1 = 0.28067f, cP2 = 0.22291f, cP3 = 2.1979f;
    const float aP1 = -0.0808f, aP2 = -0.44812f, aP3 = 1.1709f;
    const float bP1 = 0.36292f, bP2 = 1.8917f, bP3 = 1.8439f;
    const float cR1 = 0.80107f, cR2 = 0.97307f, cR3 = 3.4942f;
    const float aR1 = 0.58400f, aR2 = 0.37888f, aR3 = 2.6063f;
    const float bR1 = 0.01147f, bR2 = 3.7582f, bR3 = 0.49338f;
    const float inv_P = ff_div(FF{1.f, 0.f}, ff_add(FF{kMP2H, kMP2L}, two_MqF)).h;
    const float inv_R = ff_div(FF{1.f, 0.f}, ff_add(FF{kMR2H, kMR2L}, two_MqF)).h;
    const float inv_Q02 = 1.f / 0.52544f;
    const float inv_LQ = fpconv::f32(c.ph_inv_log_q02);
    const float Af = fpconv::f32(c.A), logA = fpconv::f32(c.ph_logA), a_low = fpconv::f32(c.ph_a_low);
    const float two_m2 = 2.f * c.mass2_f;
    const float invEE = inv_EF.h * inv_EF.h;
    const float yy = y * y;
    KSum S;
    float err = 0.f;
    bool edge = false;
    NOA_UNROLL_NODES
    for (int j = 0; j < 9; j++) {
        float Q2, unused;
        f_exp_split_aff(pc_h, pc_l, hd_h, hd_l, kF9XH[j], kF9XL[j], Q2, unused);
        const float invQ2 = f_rcp(Q2);
        const float x = 0.5f * Q2 * inv_Mq;
        // ALLM, dcs.hh:288-306
        const float t = log1pf(log1pf(Q2 * inv_Q02) * inv_LQ);
        const float xP = (Q2 + mP2) * inv_P;
        const float xR = (Q2 + mR2) * inv_R;
        const float lnt = logf(t);
        const float ecP = expf(cP3 * lnt), eaP = expf(aP3 * lnt);
        const float cP = cP1 - (cP1 - cP2) * ecP * f_rcp(1.f + ecP);
        const float aP = aP1 - (aP1 - aP2) * eaP * f_rcp(1.f + eaP);
        const float bP = bP1 + bP2 * expf(bP3 * lnt);
        const float cR = cR1 + cR2 * expf(cR3 * lnt);
        const float aR = aR1 + aR2 * expf(aR3 * lnt);
        const float bR = bR1 + bR2 * expf(bR3 * lnt);
        // 1 - x = (2Mq - Q2)/(2Mq), 2Mq - Q2 = D + Q2max (1 - exp(-dpQ2 (1 - t_j)/2))
        const float om = (D - Q2maxf * expm1f(-half_dp * (1.f - kF9XH[j]))) * inv_2Mq;
        const float l1x = logf(om);
        const float lxP = logf(xP), lxR = logf(xR);
        const float eP = aP * lxP + bP * l1x, eR = aR * lxR + bR * l1x;
        const float F2P = cP * expf(eP);
        const float F2R = cR * expf(eR);
        const float F2p = Q2 * f_rcp(Q2 + m02) * (F2P + F2R);
        // float error of F2: the exponents carry ~3 u of each |term|
        const float eF2 = U32 *
                              (F2P * (fabsf(aP * lxP) + fabsf(bP * l1x) + 2.f) +
                               F2R * (fabsf(aR * lxR) + fabsf(bR * l1x) + 2.f)) *
                              f_rcp(F2P + F2R) +
                          3.f * U32;
        // DRSS shadowing, dcs.hh:310-319
        float a = 1.f, ea = 0.f;
        if (x < 0.0014f)
            a = a_low;
        else if (x < 0.04f) {
            const float ex = (0.069f * (logf(x) * 0.4342944819f) + 0.097f) * logA;
            a = expf(ex);
            ea = U32 * (fabsf(ex) + 1.f);
        }
        edge |= fabsf(x - 0.0014f) <= 1e-6f * 0.0014f || fabsf(x - 0.04f) <= 1e-6f * 0.04f;
        const float F2A = 0.5f * Af * a * (2.f + x * (-1.85f + x * (2.45f + x * (-2.35f + x)))) * F2p;
        // Whitlow R, dcs.hh:322-332
        const bool low = Q2 < 0.3f;
        const float q2 = low ? 0.3f : Q2;
        const float inv_q2 = low ? 3.33333333f : invQ2;
        const float theta = 1.f + 12.f * q2 * 0.015625f * f_rcp((1.f + q2) * (0.015625f + x * x));
        const float R = 0.635f * theta * f_rcp(logf(q2 * 25.f)) + 0.5747f * inv_q2 - 0.3534f * f_rcp(0.09f + q2 * q2);
        // d2sigma, dcs.hh:348-354, without cf / q (applied in double below)
        const float T2 = 0.5f * (1.f - two_m2 * invQ2) * (yy + Q2 * invEE) * f_rcp(1.f + R);
        const float X = omy + T2;
        const float d_a = X * invQ2 * invQ2, d_b = 0.25f * invEE * invQ2;
        const float dds = d_a - d_b;
        const float g = F2A * dds * Q2;
        S.add(g * kF9W[j]);
        const float e_dds = 2.f * U32 * (fabsf(d_a) + fabsf(d_b)) +
                            fabsf(d_a) * 3.f * U32 * (fabsf(omy) + fabsf(T2)) * f_rcp(fabsf(X));
        err += kF9W[j] * (fabsf(g) * (eF2 + ea + 4.f * U32) + fabsf(F2A * Q2) * e_dds);
    }
    const double ds_f = S.value();
    est = edge ? INFINITY : 0.6f * err * f_rcp(fpconv::f32(fabs(ds_f)));  // calibrated: max error <= est
    // 0.5 ds dpQ2 cf (m + K) / q N_A 1e3 / A (dcs.hh:402-404), cf = 2.603096e-35
    const double fac = ff_to_double(ff_mul(dpQ2F, ff_div(ff_add(massF, KF), qF)));
    const double ds = ds_f * fac;
    return (ds < 0.) ? 0. : ds * c.ph_scale;
}

// ---------------------------------------------------------------- ionisation
// W_max = 2 me P2 / (m^2 + me (me + 2E)) of dcs.hh:415-419 equals
// 2 me K (K + 2m) / ((m + me)^2 + 2 me K) (E = K + m); every term is positive,
// so float-float keeps it to ~1e-13 relative.
constexpr float kTwoMeH = (float)(2. * ME);
constexpr float kTwoMeL = (float)(2. * ME - (double)kTwoMeH);

// The reference's three zero conditions (dcs.hh:420-424) are decided from a
// float-float W_max where they are clear by a relative margin of 1e-5, and by
// the FP64 redo (est = infinity) inside the margin, so the zero pattern is
// the reference's.  q <= 0.62 I is an exact integer compare of bit patterns.
//
// The close-collision cross-section's a1 + a2/q cancels by up to gamma^2 near
// q = W_max as the reference writes it (dcs.hh:427-431); rearranged into
// non-negative terms it runs in FP32, with W_max - q from the float-float
// W_max (q >= 1e-5 below it, so to ~1e-8 relative).  The radiative
// correction, a relative term of O(1e-2), is FP32, with E - q in float-float.
NOA_HD double ion_fp32c(double K, double q, const noa_dcs_consts &c, float &est) {
    est = 0.f;
    const long long qb = dbits(q);
    if (qb >= 0 && qb <= dbits(c.io_Wmin))  // +0 <= q <= Wmin
        return 0.;
    const float Kf = fpconv::f32(K), qf = fpconv::f32(q);
    if (!(Kf > 1e-20f && Kf < 1e12f && qf > 1e-20f && qf < 1e12f)) {  // NaN, q < 0, extreme ranges
        est = INFINITY;
        return 0.;
    }
    const FF Kx = ff_split(K), qx = ff_split(q);
    const FF two_me{kTwoMeH, kTwoMeL};
    const FF P2 = ff_mul(Kx, ff_add(Kx, FF{2.f * c.mass_h, 2.f * c.mass_l}));
    const FF W = ff_div(ff_mul(two_me, P2), ff_add(FF{c.io_cm_h, c.io_cm_l}, ff_mul(two_me, Kx)));
    const FF dW = ff_add(W, ff_neg(qx));
    constexpr float margin = 1e-5f;
    const float XK = (float)NOA_X_FRACTION * Kf;
    if (W.h < XK * (1.f - margin) || dW.h < -margin * qf)  // W_max < X K, or q > W_max
        return 0.;
    if (!(W.h > XK * (1.f + margin) && dW.h > margin * qf)) {  // within the margin of a bound
        est = INFINITY;
        return 0.;
    }
    // Close-collision term, dcs.hh:427-431, rearranged so that every term is
    // non-negative for q <= W_max (E^2 = P2 + m^2):
    //   a0 + (a1 + a2/q)/q = 0.5/P2 + ((W_max - q)/(q W_max) + m^2/(P2 q))/q.
    const float iq = f_rcp(qf), iP2 = f_rcp(P2.h);
    const float bracket = 0.5f * iP2 + iq * (dW.h * iq * f_rcp(W.h) + c.mass2_f * iP2 * iq);
    // E and E - q in float-float (E - q >= m: no cancellation beyond E / m)
    const FF EF = ff_add(Kx, FF{c.mass_h, c.mass_l});
    const float Ef = EF.h;
    float cs = fpconv::f32(c.io_cZA) * Ef * bracket;
    float Delta = 0.f;
    if (dbits(K) >= dbits(c.io_k_rad)) {  // K >= k_rad, both positive
        const float L1 = log1pf(qf * (float)(2. / ME));
        const FF Emq = ff_add(EF, ff_neg(qx));
        Delta = 1.16141E-03f * L1 * (logf(4.f * Ef * (Emq.h + Emq.l) * fpconv::f32(c.inv_m2)) - L1);
        cs *= 1.f + Delta;
    }
    // the close-collision term (max observed 8.7 u) and Delta relative to 1 + Delta
    est = (13.f + fabsf(Delta) * 8.f) * U32;
    return fpconv::f64(cs);
}

} // namespace noa_dcs
