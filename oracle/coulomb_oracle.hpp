/*
 * CPU oracle for NOA's elastic (Coulomb) scattering and transverse-transport
 * functions -- TEST INFRASTRUCTURE ONLY.
 *
 * Scalar restatement, in the reference's operation order (so that compiled
 * with -ffp-contract=off it reproduces the reference's CPU output bit for
 * bit), of:
 *   coulomb_frame_parameters / coulomb_spin_factor / coulomb_wentzel_path /
 *   coulomb_screening_parameters / coulomb_data            dcs.hh:499-622
 *   coulomb_transport_coefficients / coulomb_transport     dcs.hh:624-699
 *   coulomb_restricted_cs / cutoff_objective               dcs.hh:702-752
 *   coulomb_hard_scattering / hard_scattering              dcs.hh:754-872
 *   ridders_root                                           numerics.hh:154-216
 *   transverse_transport_ionisation / _photonuclear /
 *   soft_scattering                                        dcs.hh:874-952
 * It checks the CUDA kernels in noa_gb300/csrc/coulomb.cu and the soft
 * scattering kernel of noa_gb300/csrc/dcs_integral.cu.
 */
#pragma once

#include "dcs_oracle.hpp"

#include <algorithm>
#include <cmath>
#include <cstdint>

namespace noa_oracle {

// physics.hh:55, 78-87
constexpr double ATOMIC_MASS_ENERGY = 0.931494;
constexpr double KIN_CUTOFF = 1E-9;
constexpr double EHS_PATH_MAX = 1E+9;
constexpr double EHS_OVER_MSC = 1E-4;
constexpr int NSF = 9;

// physics.hh:83-84: half of (1 - cos) of the 1 degree maximum soft angle.
inline double max_mu0() { return 0.5 * (1. - std::cos(1E+00 * M_PI / 180.)); }

// dcs.hh:499-522: centre-of-mass Lorentz factors fCM[0..1]; returns the
// kinetic energy in the CM frame, floored at KIN_CUTOFF.
inline double coulomb_frame_parameters(double *fCM, double K, const Element &el, double mass) {
    const double Ma = el.A * ATOMIC_MASS_ENERGY;
    double M2 = mass + Ma;
    M2 *= M2;
    const double sCM12i = 1. / std::sqrt(M2 + 2. * Ma * K);
    fCM[0] = (K + mass + Ma) * sCM12i;
    double kinetic0 = (K * Ma + mass * (mass + Ma)) * sCM12i - mass;
    if (kinetic0 < KIN_CUTOFF)
        kinetic0 = KIN_CUTOFF;
    const double etot = K + mass + Ma;
    const double betaCM2 = K * (K + 2. * mass) / (etot * etot);
    double rM2 = mass / Ma;
    rM2 *= rM2;
    fCM[1] = std::sqrt(rM2 * (1. - betaCM2) + betaCM2);
    return kinetic0;
}

// dcs.hh:525-528
inline double coulomb_spin_factor(double K, double mass) {
    const double e = K + mass;
    return K * (e + mass) / (e * e);
}

// dcs.hh:531-538
inline double coulomb_wentzel_path(double screening, double K, const Element &el, double mass) {
    const double d = K * (K + 2. * mass) / (el.Z * (K + mass));
    return el.A * 2.54910918E+08 * screening * (1. + screening) * d * d;
}

// dcs.hh:541-602: atomic (Moliere with Kuraev's Coulomb correction) and two
// nuclear screening parameters, their pole-reduction factors, and the
// inverse Wentzel path.
inline double coulomb_screening_parameters(double *ps, double K, const Element &el, double mass) {
    const double third = 1. / 3;
    const double A13 = std::pow(el.A, third);
    const double R1 = 1.02934 * A13 + 0.435;
    const double R2 = 2.;
    const double p2 = K * (K + 2. * mass);
    const double d = 5.8406E-02 / p2;
    ps[1] = d / (R1 * R1);
    ps[2] = d / (R2 * R2);

    const int32_t Z = el.Z;
    const double etot = K + mass;
    const double ZE = Z * etot;
    const double zeta2 = 5.3251346E-05 * (ZE * ZE) / p2;
    double cK;
    if (zeta2 > 1.) {
        const int32_t n = 10 + Z;
        double f = 0.;
        for (int32_t i = 1; i <= n; i++)
            f += zeta2 / (i * (i * i + zeta2));
        cK = std::exp(f);
    } else {
        cK = std::exp(1. - 1. / (1. + zeta2) + zeta2 * (0.2021 + zeta2 * (0.0083 * zeta2 - 0.0369)));
    }
    const double cM = 1. + 3.34 * zeta2;
    double r = K / etot;
    r *= r;
    const double c = r * cK + (1. - r) * cM;
    ps[0] = 5.179587126E-12 * std::pow(double(Z), 2. / 3.) * c / p2;

    const double d01 = 1. / (ps[0] - ps[1]);
    const double d02 = 1. / (ps[0] - ps[2]);
    const double d12 = 1. / (ps[1] - ps[2]);
    ps[6] = d01 * d01 * d02 * d02;
    ps[7] = d01 * d01 * d12 * d12;
    ps[8] = d12 * d12 * d02 * d02;
    ps[3] = 2. * ps[6] * (d01 + d02);
    ps[4] = 2. * ps[7] * (d12 - d01);
    ps[5] = -2. * ps[8] * (d12 + d02);
    return 1. / coulomb_wentzel_path(ps[0], K, el, mass);
}

// dcs.hh:604-622 for one kinetic energy.
inline void coulomb_data(double *fCM, double *screen, double *fspin, double *invlambda, double K,
                         const Element &el, double mass) {
    const double kinetic0 = coulomb_frame_parameters(fCM, K, el, mass);
    *fspin = coulomb_spin_factor(kinetic0, mass);
    *invlambda = coulomb_screening_parameters(screen, kinetic0, el, mass);
}

// dcs.hh:624-677: first two transport coefficients below the cut-off mu.
inline void coulomb_transport_coefficients(double *coefs, const double *ps, double fspin, double mu) {
    const double nuclear_screening = (ps[1] < ps[2]) ? ps[1] : ps[2];
    if (mu < 1E-08 * nuclear_screening) {
        const double L = std::log(1. + mu / ps[0]);
        const double r = mu / (mu + ps[0]);
        const double k = ps[0] * (1. + ps[0]);
        coefs[0] = k * (r / ps[0] - fspin * (L - r));
        const double I2 = mu - ps[0] * (r - 2. * L);
        coefs[1] = 2. * k * (L - r - fspin * I2);
        return;
    }
    double I0[3], I1[3], I2[3], J0[3], J1[3], J2[3];
    const double mu2 = 0.5 * mu * mu;
    for (int i = 0; i < 3; i++) {
        double r = mu / (mu + ps[i]);
        double L = std::log(1. + mu / ps[i]);
        double mu1 = mu;
        I0[i] = r / ps[i];
        J0[i] = L;
        I1[i] = L - r;
        r *= ps[i];
        L *= ps[i];
        J1[i] = mu1 - L;
        I2[i] = mu1 - 2. * L + r;
        L *= ps[i];
        mu1 *= ps[i];
        J2[i] = mu2 + L - mu1;
    }
    const double k = ps[0] * (1. + ps[0]) * ps[1] * ps[1] * ps[2] * ps[2];
    coefs[0] = coefs[1] = 0.;
    for (int i = 0; i < 3; i++) {
        coefs[0] += ps[3 + i] * (J0[i] - fspin * J1[i]) + ps[6 + i] * (I0[i] - fspin * I1[i]);
        coefs[1] += ps[3 + i] * (J1[i] - fspin * J2[i]) + ps[6 + i] * (I1[i] - fspin * I2[i]);
    }
    coefs[0] *= k;
    coefs[1] *= 2. * k;
}

// dcs.hh:702-740: elastic cross-section restricted to angles above mu.
inline double coulomb_restricted_cs(double mu, double fspin, const double *screen) {
    if (mu >= 1.)
        return 0.;
    const double nuclear_screening = (screen[1] < screen[2]) ? screen[1] : screen[2];
    if (mu < 1E-08 * nuclear_screening) {
        const double L = std::log((screen[0] + 1.) / (screen[0] + mu));
        const double r = (1. - mu) / ((screen[0] + mu) * (screen[0] + 1.));
        const double k = screen[0] * (1. + screen[0]);
        return k * (r - fspin * (L - screen[0] * r));
    }
    double I0[3], I1[3], J0[3], J1[3];
    for (int i = 0; i < 3; i++) {
        const double L = std::log((screen[i] + 1.) / (screen[i] + mu));
        const double r = (1. - mu) / ((screen[i] + mu) * (screen[i] + 1.));
        I0[i] = r;
        J0[i] = L;
        I1[i] = L - screen[i] * r;
        J1[i] = mu - screen[i] * L;
    }
    const double k = screen[0] * (1. + screen[0]) * screen[1] * screen[1] * screen[2] * screen[2];
    double cs = 0.;
    for (int i = 0; i < 3; i++)
        cs += screen[3 + i] * (J0[i] - fspin * J1[i]) + screen[6 + i] * (I0[i] - fspin * I1[i]);
    return k * cs;
}

// dcs.hh:742-752: element-summed restricted cross-section minus the target.
inline double cutoff_objective(double cs_h, double mu, const double *invlambda, const double *fspin,
                               const double *screen, int64_t nel, int64_t nkin) {
    double cs_tot = 0.;
    for (int64_t iel = 0; iel < nel; iel++) {
        const int64_t off = iel * nkin;
        cs_tot += invlambda[off] * coulomb_restricted_cs(mu, fspin[off], screen + NSF * off);
    }
    return cs_tot - cs_h;
}

// numerics.hh:154-216, Ridders' method.  Returns false where the reference
// returns an empty optional.
template <typename F>
inline bool ridders_root(double xa, double xb, const F &f, double fa, double fb, double xtol, double rtol,
                         uint32_t max_iter, double &root) {
    if (fa * fb > 0)
        return false;
    if (fa == 0) {
        root = xa;
        return true;
    }
    if (fb == 0) {
        root = xb;
        return true;
    }
    const double tol = xtol + rtol * std::min(std::abs(xa), std::abs(xb));
    double xn = 0.;
    for (uint32_t i = 0; i < max_iter; i++) {
        double dm = 0.5 * (xb - xa);
        const double xm = xa + dm;
        const double fm = f(xm);
        double sgn = (fb > fa) ? 1. : -1.;
        double dn = sgn * dm * fm / std::sqrt(fm * fm - fa * fb);
        sgn = (dn > 0.) ? 1. : -1.;
        dn = std::abs(dn);
        dm = std::abs(dm) - 0.5 * tol;
        if (dn < dm)
            dm = dn;
        xn = xm - sgn * dm;
        const double fn = f(xn);
        if (fn * fm < 0.0) {
            xa = xn;
            fa = fn;
            xb = xm;
            fb = fm;
        } else if (fn * fa < 0.0) {
            xb = xn;
            fb = fn;
        } else {
            xa = xn;
            fa = fn;
        }
        if (fn == 0.0 || std::abs(xb - xa) < tol) {
            root = xn;
            return true;
        }
    }
    return false;
}

// dcs.hh:754-837 for the kinetic energy whose element-0 entries the
// pointers address (element stride nkin).
inline void coulomb_hard_scattering(double &mu0, double &lb_h, const double *G, const double *fCM,
                                    const double *screen, const double *invlambda, const double *fspin,
                                    int64_t nel, int64_t nkin) {
    double invlb_m = 0., invlb1_m = 0.;
    double s_m_l = 0., s_m_h = 0.;
    for (int64_t iel = 0; iel < nel; iel++) {
        const int64_t off = iel * nkin;
        const double invlb = invlambda[off];
        const double scr = screen[NSF * off];
        invlb_m += invlb * G[2 * off];
        s_m_h += scr * invlb;
        s_m_l += invlb / scr;
        const double d = 1. / (fCM[2 * off] * (1. + fCM[1 + 2 * off]));
        invlb1_m += invlb * G[1 + 2 * off] * d * d;
    }
    const double lb_m = 1. / invlb_m;
    lb_h = std::min(EHS_OVER_MSC / invlb1_m, EHS_PATH_MAX);
    if (!(lb_m < lb_h)) {
        lb_h = lb_m;
        mu0 = 0;
        return;
    }
    const double s_m = (lb_h > 2. * lb_m) ? s_m_h * lb_m : 1. / (s_m_l * lb_m);
    mu0 = s_m * (lb_h - lb_m) / (s_m * lb_h + lb_m);
    const double cs_h = 1. / lb_h;
    auto objective = [&](double mu) { return cutoff_objective(cs_h, mu, invlambda, fspin, screen, nel, nkin); };
    double mu_max = std::min(4. * mu0, 1.);
    double mu_min = 0.25 * mu0;
    double fmax = objective(mu_max), fmin = 0.;
    if (fmax > 0.)
        return;  // the reference keeps the asymptotic mu0 and lb_h here
    fmin = objective(mu_min);
    if (fmin < 0.) {
        mu_max = mu_min;
        fmax = fmin;
        mu_min = 0.;
        fmin = objective(mu_min);
    }
    const double MAX_MU0 = max_mu0();
    if (mu_min < MAX_MU0) {
        mu_max = std::min(mu_max, MAX_MU0);
        double root;
        if (ridders_root(mu_min, mu_max, objective, fmin, fmax, 1E-6 * mu0, 1E-6, 100, root))
            mu0 = root;
    }
    mu0 = std::min(mu0, MAX_MU0);
    lb_h = objective(mu0) + cs_h;
    lb_h = (lb_h <= 1. / EHS_PATH_MAX) ? EHS_PATH_MAX : 1. / lb_h;
}

// dcs.hh:874-899
inline double transverse_transport_ionisation(double K, const Element &el, double mass) {
    const double me = ELECTRON_MASS;
    const double momentum2 = K * (K + 2. * mass);
    const double E = K + mass;
    const double Wmax = 2. * me * momentum2 / (mass * mass + me * (me + 2. * E));
    const double W0 = 2. * momentum2 / me;
    const double mu_max = Wmax / W0;
    double mu3 = K * X_FRACTION / W0;
    if (mu3 > mu_max)
        mu3 = mu_max;
    const double mu2 = 0.62 * el.I / W0;
    if (mu2 >= mu3)
        return 0.;
    const double a0 = 0.5 * W0 / momentum2;
    const double a1 = -1. / Wmax;
    const double a2 = E * E / (W0 * momentum2);
    const double cs0 = 1.535336E-05 / el.A;
    return 2. * cs0 * el.Z * (0.5 * a0 * (mu3 * mu3 - mu2 * mu2) + a1 * (mu3 - mu2) + a2 * std::log(mu3 / mu2));
}

// The mu-integrated weight of one node of the photonuclear transverse
// transport, dcs.hh:911-936 (without the DCS factor).
inline double transverse_photonuclear_ratio(double K, double q, double mass) {
    const double E = K + mass;
    const double m02 = 0.4;
    const double q2 = q * q;
    const double tmax = 1.876544 * q;
    const double tmin = q2 * mass * mass / (E * (E - q));
    const double b1 = 1. / (1. - q2 / m02);
    const double c1 = 1. / (1. - m02 / q2);
    double L1 = b1 * std::log((q2 + tmax) / (q2 + tmin));
    double L2 = c1 * std::log((m02 + tmax) / (m02 + tmin));
    const double I0 = std::log(tmax / tmin) - L1 - L2;
    L1 *= q2;
    L2 *= m02;
    const double I1 = L1 + L2;
    L1 *= q2;
    L2 *= m02;
    const double I2 = (tmax - tmin) * (b1 * q2 + c1 * m02) - L1 - L2;
    return (I1 * tmax - I2) / ((I0 * tmax - I1) * K * (K + 2. * mass));
}

// dcs.hh:901-939: 6-node composite GL over t = log(nu / X_FRACTION) on
// [log 1e-6, 0] with at least 100 points (17 intervals), times 2.
inline double transverse_transport_photonuclear(double K, const Element &el, double mass) {
    auto integrand = [&](const double &t) {
        const double nu = X_FRACTION * std::exp(t);
        const double q = nu * K;
        return photonuclear<double>(K, q, el, mass) * transverse_photonuclear_ratio(K, q, mass) * nu;
    };
    return 2. * gl_composite<double>(std::log(1E-06), 0., integrand, 100u, 6u, GL6_X, GL6_W);
}

// dcs.hh:941-952 for one kinetic energy.
inline double soft_scattering(double K, const Element &el, double mass) {
    return transverse_transport_ionisation(K, el, mass) + transverse_transport_photonuclear(K, el, mass);
}

} // namespace noa_oracle
