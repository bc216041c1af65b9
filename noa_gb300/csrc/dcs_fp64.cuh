/*
 * FP64 device functions of the four muon DCS processes.
 *
 * Each function keeps the reference's operation order inside one evaluation;
 * what depends only on (element, mass) comes precomputed in noa_dcs_consts
 * (dcs_consts.h).  Every early exit of the reference is kept with the same
 * predicate, so NaN inputs propagate as they do on the CPU.
 *
 *   bremsstrahlung   physics.hh:114-153
 *   pair production  dcs.hh:144-258, 8-node GL numerics.hh:110-129
 *   photonuclear     dcs.hh:261-405, 9-node GL numerics.hh:131-152
 *   ionisation       dcs.hh:408-443
 *
 * The `*_live` predicates evaluate only the kinematic bounds of a process
 * (the reference's early returns) so that a kernel can drop the pairs whose
 * DCS is exactly zero before running the quadrature.  Bound expressions use
 * the __d*_rn intrinsics, which the compiler never fuses into an FMA, so the
 * zero / non-zero decision rounds exactly as the reference's (unfused) CPU
 * code does, also for pairs placed exactly on a bound.
 */
#pragma once

#include "dcs_consts.h"

namespace noa_dcs {

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

constexpr double ME = NOA_ELECTRON_MASS;
constexpr double NA = NOA_AVOGADRO_NUMBER;

// ---------------------------------------------------------------- bremsstrahlung
__device__ __forceinline__ double brems_fp64(double K, double q, const noa_dcs_consts &c) {
    const double mass = c.mass;
    const double sqrte = 1.648721271;
    const double E = K + mass;
    const double delta_factor = c.br_half_m2 / E;
    const double qe_max = E / (1. + c.br_half_m2 / (ME * E));
    const double nu = q / E;
    const double delta = delta_factor * nu / (1. - nu);
    double Phi_n = log(c.br_BZ_n * (mass + delta * c.br_Dn_sqrte_m2) / (c.br_D_n * (ME + delta * sqrte * c.br_BZ_n)));
    if (Phi_n < 0.)
        Phi_n = 0.;
    double Phi_e;
    if (q < qe_max) {
        Phi_e = log(c.br_BZe_mass / ((1. + delta * c.br_phie_factor) * (ME + delta * sqrte * c.br_BZ_e)));
        if (Phi_e < 0.)
            Phi_e = 0.;
    } else
        Phi_e = 0.;
    const double dcs = c.br_dcs_factor * (c.Zd * Phi_n + Phi_e) * (4. / 3. * (1. / nu - 1.) + nu);
    return (dcs < 0.) ? 0. : dcs * 1E+03 * NA / c.A;
}

// ---------------------------------------------------------------- pair production
// Lower end of the t-integral, argmin of dcs.hh:169-173; returns a value
// outside (0, 1) when the pair is kinematically closed.
__device__ __forceinline__ double pprod_argmin(double K, double q, const noa_dcs_consts &c) {
    const double gamma = 1. + K / c.mass;
    const double x0 = 4. * ME / q;
    const double x1 = 6. / (gamma * (gamma - q / c.mass));
    return __dadd_rn(x0, __dmul_rn(2. * (1. - x0), x1)) / __dadd_rn(1., __dmul_rn(1. - x1, sqrt(1. - x0)));
}

__device__ __forceinline__ bool pprod_live(double K, double q, const noa_dcs_consts &c) {
    if (q <= 4. * ME)
        return false;
    if (q >= K + c.pp_kmax_shift)
        return false;
    const double argmin = pprod_argmin(K, q, c);
    if ((argmin >= 1.) || (argmin <= 0.))
        return false;
    return true;
}

__device__ __forceinline__ double pprod_fp64(double K, double q, const noa_dcs_consts &c) {
    if (q <= 4. * ME)
        return 0.;
    if (q >= K + c.pp_kmax_shift)
        return 0.;
    const double mass = c.mass;
    const double nu = q / (K + mass);
    const double beta = 0.5 * nu * nu / (1. - nu);
    const double xi_factor = c.pp_half_r2 * beta;
    const double gamma = 1. + K / mass;
    const double argmin = pprod_argmin(K, q, c);
    if ((argmin >= 1.) || (argmin <= 0.))
        return 0.;
    const double tmin = log(argmin);

    double I = 0.;
#pragma unroll
    for (int j = 0; j < 8; j++) {
        const double eps = exp(kGL8X[j] * tmin);
        const double rho = 1. - eps;
        const double rho2 = rho * rho;
        const double rho21 = eps * (2. - eps);
        const double xi = xi_factor * rho21;
        const double xi_i = 1. / xi;

        double Be;
        if (xi >= 1E+03)
            Be = 0.5 * xi_i * ((3. - rho2) + 2. * beta * (1. + rho2));
        else
            Be = ((2. + rho2) * (1. + beta) + xi * (3. + rho2)) * log(1. + xi_i) + (rho21 - beta) / (1. + xi) - 3. -
                 rho2;
        const double Ye = (5. - rho2 + 4. * beta * (1. + rho2)) /
                          (2. * (1. + 3. * beta) * log(3. + xi_i) - rho2 - 2. * beta * (2. - rho2));
        const double xe = (1. + xi) * (1. + Ye);
        const double cLi = c.pp_cL / rho21;
        const double Le = log(c.pp_AZ13 * sqrt(xe) * q / (q + cLi * xe)) - 0.5 * log(1. + c.pp_cLe * xe);
        double Phi_e = Be * Le;
        if (Phi_e < 0.)
            Phi_e = 0.;

        double Bmu;
        if (xi <= 1E-03)
            Bmu = 0.5 * xi * (5. - rho2 + beta * (3. + rho2));
        else
            Bmu = ((1. + rho2) * (1. + 1.5 * beta) - xi_i * (1. + 2. * beta) * rho21) * log(1. + xi) +
                  xi * (rho21 - beta) / (1. + xi) + (1. + 2. * beta) * rho21;
        const double Ymu = (4. + rho2 + 3. * beta * (1. + rho2)) /
                           ((1. + rho2) * (1.5 + 2. * beta) * log(3. + xi) + 1. - 1.5 * rho2);
        const double xmu = (1. + xi) * (1. + Ymu);
        const double Lmu = log(c.pp_r_AZ13 * q / (c.pp_15_Z13 * (q + cLi * xmu)));
        double Phi_mu = Bmu * Lmu;
        if (Phi_mu < 0.)
            Phi_mu = 0.;
        const double f = -(Phi_e + Phi_mu / c.pp_r2) * (1. - rho) * tmin;
        I += f * kGL8W[j];
    }

    double zeta;
    if (gamma <= 35.)
        zeta = 0.;
    else {
        zeta = 0.073 * log(gamma / (1. + c.pp_gamma1 * gamma * c.pp_Z13 * c.pp_Z13)) - 0.26;
        if (zeta <= 0.)
            zeta = 0.;
        else
            zeta /= 0.058 * log(gamma / (1. + c.pp_gamma2 * gamma * c.pp_Z13)) - 0.14;
    }
    const double E = K + mass;
    const double dcs = c.pp_cZ * (c.Zd + zeta) * (E - q) * I / (q * E);
    return (dcs < 0.) ? 0. : dcs * 1E+03 * NA * (mass + K) / c.A;
}

// ---------------------------------------------------------------- photonuclear
constexpr double PH_M = 0.931494;
constexpr double PH_MPI = 0.134977;

// ALLM F2, dcs.hh:261-307.
__device__ __forceinline__ double ph_f2_allm(double x, double Q2, double log_q02) {
    const double m02 = 0.31985, mP2 = 49.457, mR2 = 0.15052, Q02 = 0.52544, Lambda2 = 0.06527;
    const double cP1 = 0.28067, cP2 = 0.22291, cP3 = 2.1979;
    const double aP1 = -0.0808, aP2 = -0.44812, aP3 = 1.1709;
    const double bP1 = 0.36292, bP2 = 1.8917, bP3 = 1.8439;
    const double cR1 = 0.80107, cR2 = 0.97307, cR3 = 3.4942;
    const double aR1 = 0.58400, aR2 = 0.37888, aR3 = 2.6063;
    const double bR1 = 0.01147, bR2 = 3.7582, bR3 = 0.49338;
    const double M2 = 0.8803505929;
    const double W2 = M2 + Q2 * (1.0 / x - 1.0);
    const double t = log(log((Q2 + Q02) / Lambda2) / log_q02);
    const double xP = (Q2 + mP2) / (Q2 + mP2 + W2 - M2);
    const double xR = (Q2 + mR2) / (Q2 + mR2 + W2 - M2);
    const double lnt = log(t);
    const double cP = cP1 + (cP1 - cP2) * (1.0 / (1.0 + exp(cP3 * lnt)) - 1.0);
    const double aP = aP1 + (aP1 - aP2) * (1.0 / (1.0 + exp(aP3 * lnt)) - 1.0);
    const double bP = bP1 + bP2 * exp(bP3 * lnt);
    const double cR = cR1 + cR2 * exp(cR3 * lnt);
    const double aR = aR1 + aR2 * exp(aR3 * lnt);
    const double bR = bR1 + bR2 * exp(bR3 * lnt);
    const double l1x = log(1 - x);
    const double F2P = cP * exp(aP * log(xP) + bP * l1x);
    const double F2R = cR * exp(aR * log(xR) + bR * l1x);
    return Q2 / (Q2 + m02) * (F2P + F2R);
}

// Photonuclear DCS kinematic window, dcs.hh:357-381.  Returns false when the
// reference returns 0 before its quadrature.
__device__ __forceinline__ bool photo_live(double K, double q, const noa_dcs_consts &c) {
    if ((q < 1.) || (q < 2E-03 * K))
        return false;
    const double mass = c.mass;
    const double E = K + mass;
    if ((q >= (E - mass)) || (q <= c.ph_q_min))
        return false;
    const double y = q / E;
    const double Q2min = mass * mass * y * y / (1 - y);
    const double Q2max = __dsub_rn(__dmul_rn(2.0 * PH_M, q - PH_MPI), PH_MPI * PH_MPI);
    if ((Q2max < Q2min) | (Q2min < 0))
        return false;
    return true;
}

__device__ __forceinline__ double photo_fp64(double K, double q, const noa_dcs_consts &c) {
    if ((q < 1.) || (q < 2E-03 * K))
        return 0.;
    const double mass = c.mass;
    const double E = K + mass;
    if ((q >= (E - mass)) || (q <= c.ph_q_min))
        return 0.;
    const double y = q / E;
    const double Q2min = mass * mass * y * y / (1 - y);
    const double Q2max = __dsub_rn(__dmul_rn(2.0 * PH_M, q - PH_MPI), PH_MPI * PH_MPI);
    if ((Q2max < Q2min) | (Q2min < 0))
        return 0.;
    const double pQ2min = log(Q2min);
    const double pQ2max = log(Q2max);
    const double dpQ2 = pQ2max - pQ2min;
    const double pQ2c = 0.5 * (pQ2max + pQ2min);

    // d2sigma/dQ2 pieces that do not depend on Q2, dcs.hh:338-343.
    const double cf = 2.603096E-35;
    const double EE = E * E;
    const double Mq = PH_M * q;
    const double two_m2 = 2 * mass * mass;
    double ds = 0.;
#pragma unroll 1
    for (int j = 0; j < 9; j++) {
        const double Q2 = exp(pQ2c + 0.5 * dpQ2 * kGL9X[j]);
        const double x = 0.5 * Q2 / Mq;
        const double F2p = ph_f2_allm(x, Q2, c.ph_log_q02);
        // DRSS shadowing, dcs.hh:310-319.
        double a = 1.0;
        if (x < 0.0014)
            a = c.ph_a_low;
        else if (x < 0.04)
            a = exp((0.069 * log10(x) + 0.097) * c.ph_logA);
        const double F2A = (0.5 * c.A * a * (2.0 + x * (-1.85 + x * (2.45 + x * (-2.35 + x)))) * F2p);
        // Whitlow R, dcs.hh:322-332.
        double q2 = Q2;
        if (Q2 < 0.3)
            q2 = 0.3;
        const double theta = 1 + 12.0 * q2 / (1.0 + q2) * 0.015625 / (0.015625 + x * x);
        const double R = (0.635 / log(q2 / 0.04) * theta + 0.5747 / q2 - 0.3534 / (0.09 + q2 * q2));
        // dcs.hh:348-354.
        const double dds = (1 - y + 0.5 * (1 - two_m2 / Q2) * (y * y + Q2 / EE) / (1 + R)) / (Q2 * Q2) -
                           0.25 / (EE * Q2);
        const double d2 = cf * F2A * dds / q;
        ds += d2 * Q2 * kGL9W[j];
    }
    return (ds < 0.) ? 0. : 0.5 * ds * dpQ2 * 1E+03 * NA * (mass + K) / c.A;
}

// ---------------------------------------------------------------- ionisation
__device__ __forceinline__ double ion_fp64(double K, double q, const noa_dcs_consts &c) {
    const double mass = c.mass;
    const double P2 = K * (K + 2. * mass);
    const double E = K + mass;
    const double Wmax = 2. * ME * P2 / __dadd_rn(__dmul_rn(mass, mass), __dmul_rn(ME, ME + 2. * E));
    if ((Wmax < NOA_X_FRACTION * K) || (q > Wmax))
        return 0.;
    if (q <= c.io_Wmin)
        return 0.;
    const double a0 = 0.5 / P2;
    const double a1 = -1. / Wmax;
    const double a2 = E * E / P2;
    const double cs = 1.535336E-05 * E * c.Zd / c.A * (a0 + 1. / q * (a1 + a2 / q));
    double Delta = 0.;
    if (K >= c.io_k_rad) {
        const double L1 = log(1. + 2. * q / ME);
        Delta = 1.16141E-03 * L1 * (log(4. * E * (E - q) / (mass * mass)) - L1);
    }
    return cs * (1. + Delta);
}

} // namespace noa_dcs
