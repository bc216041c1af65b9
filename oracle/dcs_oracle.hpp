/*
 * CPU oracle for the NOA PMS muon DCS hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * This header restates, in scalar C++, the four differential cross-sections of
 * NOA (grinisrit/noa) in the reference's operation order, so that compiled
 * with IEEE semantics (-O2 -ffp-contract=off, no fast-math) it reproduces the
 * reference's own CPU output bit for bit.  The tests compare the CUDA
 * kernels in noa_gb300/csrc with it; it is never linked into the product
 * library.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline use it.
 *
 * Every function is templated on the scalar type so that the same source can
 * be instantiated with an operation-counting scalar (dcs_opcount.cpp) to give
 * the algorithmic work per evaluation.
 *
 * Reference files (paths relative to the grinisrit/noa repository root):
 *   src/noa/pms/physics.hh   constants, AtomicElement, _bremsstrahlung_
 *   src/noa/pms/dcs.hh       pair_production, photonuclear (+ALLM/DRSS/Whitlow), ionisation,
 *                            recoil_integral, analytic ionisation integrals
 *   src/noa/utils/numerics.hh  Gauss-Legendre tables and the composite driver
 */
#pragma once

#include <cmath>
#include <cstdint>

namespace noa_oracle {

// physics.hh:54-58
constexpr double AVOGADRO_NUMBER = 6.02214076E+23;
constexpr double ELECTRON_MASS = 0.510998910E-03;
constexpr double MUON_MASS = 0.10565839;
// physics.hh:76
constexpr double X_FRACTION = 5E-02;

// Mirrors noa::pms::AtomicElement (physics.hh:39-43): {A g/mol, I GeV, Z}.
struct Element {
    double A;
    double I;
    int32_t Z;
};

// Gauss-Legendre tables exactly as the reference literals (numerics.hh:97-100,
// 116-121, 137-144).  The 6- and 8-node tables are 8-digit truncations on
// [0,1]; the 9-node table is on [-1,1].  Parity needs these literals, not the
// exact nodes.
constexpr double GL6_X[6] = {0.03376524, 0.16939531, 0.38069041, 0.61930959, 0.83060469, 0.96623476};
constexpr double GL6_W[6] = {0.08566225, 0.18038079, 0.23395697, 0.23395697, 0.18038079, 0.08566225};
constexpr double GL8_X[8] = {0.01985507, 0.10166676, 0.2372338, 0.40828268,
                             0.59171732, 0.7627662, 0.89833324, 0.98014493};
constexpr double GL8_W[8] = {0.05061427, 0.11119052, 0.15685332, 0.18134189,
                             0.18134189, 0.15685332, 0.11119052, 0.05061427};
constexpr double GL9_X[9] = {0.0000000000000000, -0.8360311073266358, 0.8360311073266358,
                             -0.9681602395076261, 0.9681602395076261, -0.3242534234038089,
                             0.3242534234038089, -0.6133714327005904, 0.6133714327005904};
constexpr double GL9_W[9] = {0.3302393550012598, 0.1806481606948574, 0.1806481606948574,
                             0.0812743883615744, 0.0812743883615744, 0.3123470770400029,
                             0.3123470770400029, 0.2606106964029354, 0.2606106964029354};

// Composite Gauss-Legendre driver, numerics.hh:71-89: n_itv = ceil(min_points/order)
// intervals of width h; the sum runs node by node in one accumulator, each
// term formed as f(x) * h * w.
template <typename R, typename F>
inline R gl_composite(R lo, R hi, const F &f, uint32_t min_points, uint32_t order,
                      const double *xs, const double *ws) {
    const uint32_t n_itv = (min_points + order - 1) / order;
    const R h = (hi - lo) / R(double(n_itv));
    const uint32_t N = n_itv * order;
    R res = R(0.0);
    for (uint32_t i = 0; i < N; i++) {
        const uint32_t j = i % order;
        res += f(lo + h * (R(double(i / order)) + R(xs[j]))) * h * R(ws[j]);
    }
    return res;
}

// physics.hh:114-153 (_bremsstrahlung_).
template <typename R>
inline R bremsstrahlung(R kinetic_energy, R recoil_energy, const Element &el, double mass_) {
    using std::log;
    using std::pow;
    const int32_t Z = el.Z;
    const R A = R(el.A);
    const R mass = R(mass_);
    const R me = R(ELECTRON_MASS);
    const R sqrte = R(1.648721271);
    const R phie_factor = mass / (me * me * sqrte);
    const R rem = R(5.63588E-13) * me / mass;

    const R BZ_n = (Z == 1) ? R(202.4) : R(182.7) * pow(R(double(Z)), R(-1. / 3.));
    const R BZ_e = (Z == 1) ? R(446.) : R(1429.) * pow(R(double(Z)), R(-2. / 3.));
    const R D_n = R(1.54) * pow(A, R(0.27));
    const R E = kinetic_energy + mass;
    const R dcs_factor = R(7.297182E-07) * rem * rem * R(double(Z));

    const R delta_factor = R(0.5) * mass * mass / E;
    const R qe_max = E / (R(1.) + R(0.5) * mass * mass / (me * E));

    const R nu = recoil_energy / E;
    const R delta = delta_factor * nu / (R(1.) - nu);
    R Phi_n, Phi_e;
    Phi_n = log(BZ_n * (mass + delta * (D_n * sqrte - R(2.))) / (D_n * (me + delta * sqrte * BZ_n)));
    if (Phi_n < R(0.))
        Phi_n = R(0.);
    if (recoil_energy < qe_max) {
        Phi_e = log(BZ_e * mass / ((R(1.) + delta * phie_factor) * (me + delta * sqrte * BZ_e)));
        if (Phi_e < R(0.))
            Phi_e = R(0.);
    } else
        Phi_e = R(0.);

    const R dcs = dcs_factor * (R(double(Z)) * Phi_n + Phi_e) * (R(4. / 3.) * (R(1.) / nu - R(1.)) + nu);
    return (dcs < R(0.)) ? R(0.) : dcs * R(1E+03) * R(AVOGADRO_NUMBER) / A;
}

// dcs.hh:144-258 (pair_production): bounds, then one 8-node GL over
// t in [0,1] with rho = 1 - exp(t * tmin), then the atomic-electron form factor.
template <typename R>
inline R pair_production(R kinetic_energy, R recoil_energy, const Element &el, double mass_) {
    using std::exp;
    using std::log;
    using std::pow;
    using std::sqrt;
    const int32_t Z = el.Z;
    const R A = R(el.A);
    const R mass = R(mass_);
    const R Zd = R(double(Z));
    if (recoil_energy <= R(4.) * R(ELECTRON_MASS))
        return R(0.);
    const R sqrte = R(1.6487212707);
    const R Z13 = pow(Zd, R(1. / 3.));
    if (recoil_energy >= kinetic_energy + mass * (R(1.) - R(0.75) * sqrte * Z13))
        return R(0.);

    const R nu = recoil_energy / (kinetic_energy + mass);
    const R r = mass / R(ELECTRON_MASS);
    const R beta = R(0.5) * nu * nu / (R(1.) - nu);
    const R xi_factor = R(0.5) * r * r * beta;
    const R A_ = (Z == 1) ? R(202.4) : R(183.);
    const R AZ13 = A_ / Z13;
    const R cL = R(2.) * sqrte * R(ELECTRON_MASS) * AZ13;
    const R cLe = R(2.25) * Z13 * Z13 / (r * r);

    const R gamma = R(1.) + kinetic_energy / mass;
    const R x0 = R(4.) * R(ELECTRON_MASS) / recoil_energy;
    const R x1 = R(6.) / (gamma * (gamma - recoil_energy / mass));
    const R argmin = (x0 + R(2.) * (R(1.) - x0) * x1) / (R(1.) + (R(1.) - x1) * sqrt(R(1.) - x0));
    if ((argmin >= R(1.)) || (argmin <= R(0.)))
        return R(0.);
    const R tmin = log(argmin);

    auto integrand = [&](const R &t) {
        const R eps = exp(t * tmin);
        const R rho = R(1.) - eps;
        const R rho2 = rho * rho;
        const R rho21 = eps * (R(2.) - eps);
        const R xi = xi_factor * rho21;
        const R xi_i = R(1.) / xi;

        R Be;
        if (xi >= R(1E+03))
            Be = R(0.5) * xi_i * ((R(3.) - rho2) + R(2.) * beta * (R(1.) + rho2));
        else
            Be = ((R(2.) + rho2) * (R(1.) + beta) + xi * (R(3.) + rho2)) * log(R(1.) + xi_i) +
                 (rho21 - beta) / (R(1.) + xi) - R(3.) - rho2;
        const R Ye = (R(5.) - rho2 + R(4.) * beta * (R(1.) + rho2)) /
                     (R(2.) * (R(1.) + R(3.) * beta) * log(R(3.) + xi_i) - rho2 - R(2.) * beta * (R(2.) - rho2));
        const R xe = (R(1.) + xi) * (R(1.) + Ye);
        const R cLi = cL / rho21;
        const R Le = log(AZ13 * sqrt(xe) * recoil_energy / (recoil_energy + cLi * xe)) -
                     R(0.5) * log(R(1.) + cLe * xe);
        R Phi_e = Be * Le;
        if (Phi_e < R(0.))
            Phi_e = R(0.);

        R Bmu;
        if (xi <= R(1E-03))
            Bmu = R(0.5) * xi * (R(5.) - rho2 + beta * (R(3.) + rho2));
        else
            Bmu = ((R(1.) + rho2) * (R(1.) + R(1.5) * beta) - xi_i * (R(1.) + R(2.) * beta) * rho21) *
                          log(R(1.) + xi) +
                  xi * (rho21 - beta) / (R(1.) + xi) + (R(1.) + R(2.) * beta) * rho21;
        const R Ymu = (R(4.) + rho2 + R(3.) * beta * (R(1.) + rho2)) /
                      ((R(1.) + rho2) * (R(1.5) + R(2.) * beta) * log(R(3.) + xi) + R(1.) - R(1.5) * rho2);
        const R xmu = (R(1.) + xi) * (R(1.) + Ymu);
        const R Lmu = log(r * AZ13 * recoil_energy / (R(1.5) * Z13 * (recoil_energy + cLi * xmu)));
        R Phi_mu = Bmu * Lmu;
        if (Phi_mu < R(0.))
            Phi_mu = R(0.);
        return -(Phi_e + Phi_mu / (r * r)) * (R(1.) - rho) * tmin;
    };
    const R I = gl_composite<R>(R(0.0), R(1.0), integrand, 1u, 8u, GL8_X, GL8_W);

    R zeta;
    if (gamma <= R(35.))
        zeta = R(0.);
    else {
        R gamma1, gamma2;
        if (Z == 1) {
            gamma1 = R(4.4E-05);
            gamma2 = R(4.8E-05);
        } else {
            gamma1 = R(1.95E-05);
            gamma2 = R(5.30E-05);
        }
        zeta = R(0.073) * log(gamma / (R(1.) + gamma1 * gamma * Z13 * Z13)) - R(0.26);
        if (zeta <= R(0.))
            zeta = R(0.);
        else
            zeta /= R(0.058) * log(gamma / (R(1.) + gamma2 * gamma * Z13)) - R(0.14);
    }

    const R E = kinetic_energy + mass;
    const R dcs = R(1.794664E-34) * Zd * (Zd + zeta) * (E - recoil_energy) * I / (recoil_energy * E);
    return (dcs < R(0.)) ? R(0.) : dcs * R(1E+03) * R(AVOGADRO_NUMBER) * (mass + kinetic_energy) / A;
}

// dcs.hh:261-307, ALLM proton structure function F2(x, Q2).
template <typename R>
inline R photonuclear_f2_allm(R x, R Q2) {
    using std::exp;
    using std::log;
    const R m02 = R(0.31985), mP2 = R(49.457), mR2 = R(0.15052), Q02 = R(0.52544), Lambda2 = R(0.06527);
    const R cP1 = R(0.28067), cP2 = R(0.22291), cP3 = R(2.1979);
    const R aP1 = R(-0.0808), aP2 = R(-0.44812), aP3 = R(1.1709);
    const R bP1 = R(0.36292), bP2 = R(1.8917), bP3 = R(1.8439);
    const R cR1 = R(0.80107), cR2 = R(0.97307), cR3 = R(3.4942);
    const R aR1 = R(0.58400), aR2 = R(0.37888), aR3 = R(2.6063);
    const R bR1 = R(0.01147), bR2 = R(3.7582), bR3 = R(0.49338);
    const R M2 = R(0.8803505929);
    const R W2 = M2 + Q2 * (R(1.0) / x - R(1.0));
    const R t = log(log((Q2 + Q02) / Lambda2) / log(Q02 / Lambda2));
    const R xP = (Q2 + mP2) / (Q2 + mP2 + W2 - M2);
    const R xR = (Q2 + mR2) / (Q2 + mR2 + W2 - M2);
    const R lnt = log(t);
    const R cP = cP1 + (cP1 - cP2) * (R(1.0) / (R(1.0) + exp(cP3 * lnt)) - R(1.0));
    const R aP = aP1 + (aP1 - aP2) * (R(1.0) / (R(1.0) + exp(aP3 * lnt)) - R(1.0));
    const R bP = bP1 + bP2 * exp(bP3 * lnt);
    const R cR = cR1 + cR2 * exp(cR3 * lnt);
    const R aR = aR1 + aR2 * exp(aR3 * lnt);
    const R bR = bR1 + bR2 * exp(bR3 * lnt);
    const R F2P = cP * exp(aP * log(xP) + bP * log(R(1.) - x));
    const R F2R = cR * exp(aR * log(xR) + bR * log(R(1.) - x));
    return Q2 / (Q2 + m02) * (F2P + F2R);
}

// dcs.hh:310-319, DRSS nuclear shadowing.
template <typename R>
inline R photonuclear_f2a_drss(R x, R F2p, double A_) {
    using std::exp;
    using std::log;
    using std::log10;
    const R A = R(A_);
    R a = R(1.0);
    if (x < R(0.0014))
        a = exp(R(-0.1) * log(A));
    else if (x < R(0.04))
        a = exp((R(0.069) * log10(x) + R(0.097)) * log(A));
    return (R(0.5) * A * a * (R(2.0) + x * (R(-1.85) + x * (R(2.45) + x * (R(-2.35) + x)))) * F2p);
}

// dcs.hh:322-332, Whitlow R = sigma_L / sigma_T.
template <typename R>
inline R photonuclear_r_whitlow(R x, R Q2) {
    using std::log;
    R q2 = Q2;
    if (Q2 < R(0.3))
        q2 = R(0.3);
    const R theta = R(1.) + R(12.0) * q2 / (R(1.0) + q2) * R(0.015625) / (R(0.015625) + x * x);
    return (R(0.635) / log(q2 / R(0.04)) * theta + R(0.5747) / q2 - R(0.3534) / (R(0.09) + q2 * q2));
}

// dcs.hh:335-355, doubly differential cross-section d2sigma/(dq dQ2).
template <typename R>
inline R photonuclear_d2(double A, double mass_, R kinetic_energy, R recoil_energy, R Q2) {
    const R mass = R(mass_);
    const R cf = R(2.603096E-35);
    const R M = R(0.931494);
    const R E = kinetic_energy + mass;
    const R y = recoil_energy / E;
    const R x = R(0.5) * Q2 / (M * recoil_energy);
    const R F2p = photonuclear_f2_allm<R>(x, Q2);
    const R F2A = photonuclear_f2a_drss<R>(x, F2p, A);
    const R R_ = photonuclear_r_whitlow<R>(x, Q2);
    const R dds = (R(1.) - y + R(0.5) * (R(1.) - R(2.) * mass * mass / Q2) * (y * y + Q2 / (E * E)) / (R(1.) + R_)) /
                          (Q2 * Q2) -
                  R(0.25) / (E * E * Q2);
    return cf * F2A * dds / recoil_energy;
}

// dcs.hh:362-405 (photonuclear): cuts, then a 9-node GL over log Q2.
template <typename R>
inline R photonuclear(R kinetic_energy, R recoil_energy, const Element &el, double mass_) {
    using std::exp;
    using std::log;
    // dcs_photonuclear_check, dcs.hh:357-359
    if ((recoil_energy < R(1.)) || (recoil_energy < R(2E-03) * kinetic_energy))
        return R(0.);
    const double A = el.A;
    const R mass = R(mass_);
    const R M = R(0.931494);
    const R mpi = R(0.134977);
    const R E = kinetic_energy + mass;
    if ((recoil_energy >= (E - mass)) || (recoil_energy <= (mpi * (R(1.0) + R(0.5) * mpi / M))))
        return R(0.);
    const R y = recoil_energy / E;
    const R Q2min = mass * mass * y * y / (R(1) - y);
    const R Q2max = R(2.0) * M * (recoil_energy - mpi) - mpi * mpi;
    if ((Q2max < Q2min) || (Q2min < R(0)))
        return R(0.);
    const R pQ2min = log(Q2min);
    const R pQ2max = log(Q2max);
    const R dpQ2 = pQ2max - pQ2min;
    const R pQ2c = R(0.5) * (pQ2max + pQ2min);
    auto integrand = [&](const R &t) {
        const R Q2 = exp(pQ2c + R(0.5) * dpQ2 * t);
        return photonuclear_d2<R>(A, mass_, kinetic_energy, recoil_energy, Q2) * Q2;
    };
    const R ds = gl_composite<R>(R(0.0), R(1.0), integrand, 1u, 9u, GL9_X, GL9_W);
    return (ds < R(0.)) ? R(0.) : R(0.5) * ds * dpQ2 * R(1E+03) * R(AVOGADRO_NUMBER) * (mass + kinetic_energy) / R(A);
}

// dcs.hh:408-443 (ionisation): close collisions plus radiative correction.
template <typename R>
inline R ionisation(R kinetic_energy, R recoil_energy, const Element &el, double mass_) {
    using std::log;
    const R A = R(el.A);
    const R Zd = R(double(el.Z));
    const R mass = R(mass_);
    const R me = R(ELECTRON_MASS);
    const R P2 = kinetic_energy * (kinetic_energy + R(2.) * mass);
    const R E = kinetic_energy + mass;
    const R Wmax = R(2.) * me * P2 / (mass * mass + me * (me + R(2.) * E));
    if ((Wmax < R(X_FRACTION) * kinetic_energy) || (recoil_energy > Wmax))
        return R(0.);
    const R Wmin = R(0.62) * R(el.I);
    if (recoil_energy <= Wmin)
        return R(0.);
    const R a0 = R(0.5) / P2;
    const R a1 = R(-1.) / Wmax;
    const R a2 = E * E / P2;
    const R cs = R(1.535336E-05) * E * Zd / A * (a0 + R(1.) / recoil_energy * (a1 + a2 / recoil_energy));
    R Delta = R(0.);
    const R m1 = mass - me;
    if (kinetic_energy >= R(0.5) * m1 * m1 / me) {
        const R L1 = log(R(1.) + R(2.) * recoil_energy / me);
        Delta = R(1.16141E-03) * L1 * (log(R(4.) * E * (E - recoil_energy) / (mass * mass)) - L1);
    }
    return cs * (R(1.) + Delta);
}

enum Process { BREMSSTRAHLUNG = 0, PAIR_PRODUCTION = 1, PHOTONUCLEAR = 2, IONISATION = 3 };

template <typename R>
inline R dcs(int process, R k, R q, const Element &el, double mass) {
    switch (process) {
    case BREMSSTRAHLUNG:
        return bremsstrahlung<R>(k, q, el, mass);
    case PAIR_PRODUCTION:
        return pair_production<R>(k, q, el, mass);
    case PHOTONUCLEAR:
        return photonuclear<R>(k, q, el, mass);
    default:
        return ionisation<R>(k, q, el, mass);
    }
}

// dcs.hh:89-105 (recoil_integral) with del_integrand (dcs*q, :107-109) or
// cel_integrand (dcs*q*q, :111-113): 6-node composite GL over t = log q on
// [log(K*xlow), log K], divided by the total energy.
template <typename R>
inline R recoil_integral(int process, int moment, R kinetic_energy, R xlow, const Element &el, double mass,
                         uint32_t min_points) {
    using std::exp;
    using std::log;
    auto integrand = [&](const R &t) {
        const R q = exp(t);
        const R d = dcs<R>(process, kinetic_energy, q, el, mass);
        return moment == 0 ? d * q : d * q * q;
    };
    return gl_composite<R>(log(kinetic_energy * xlow), log(kinetic_energy), integrand, min_points, 6u, GL6_X, GL6_W) /
           (kinetic_energy + R(mass));
}

// dcs.hh:446-496: closed forms of the ionisation DEL / CEL integrals.
template <typename R>
inline R analytic_ionisation_recoil_integral(int moment, R kinetic_energy, R xlow, const Element &el,
                                             double mass_) {
    using std::log;
    const R mass = R(mass_);
    const R me = R(ELECTRON_MASS);
    const R P2 = kinetic_energy * (kinetic_energy + R(2.) * mass);
    const R E = kinetic_energy + mass;
    const R Wmax = R(2.) * me * P2 / (mass * mass + me * (me + R(2.) * E));
    if (Wmax < R(X_FRACTION) * kinetic_energy)
        return R(0.);
    R Wmin = R(0.62) * R(el.I);
    const R qlow = kinetic_energy * xlow;
    if (qlow >= Wmin)
        Wmin = qlow;
    if (Wmax <= Wmin)
        return R(0.);
    const R a0 = R(0.5) / P2, a1 = R(-1.) / Wmax, a2 = E * E / P2;
    R term;
    if (moment == 0)
        term = a0 * (Wmax - Wmin) + a1 * log(Wmax / Wmin) + a2 * (R(1.) / Wmin - R(1.) / Wmax);
    else
        term = R(0.5) * a0 * (Wmax * Wmax - Wmin * Wmin) + a1 * (Wmax - Wmin) + a2 * log(Wmax / Wmin);
    return R(1.535336E-05) * R(double(el.Z)) / R(el.A) * term;
}

// dcs.hh:955-1001: the ionisation specialisation switches to the closed form
// below the radiative-correction threshold.
template <typename R>
inline R recoil_integral_dispatch(int process, int moment, R kinetic_energy, R xlow, const Element &el,
                                  double mass, uint32_t min_points) {
    if (process == IONISATION) {
        const R m1 = R(mass) - R(ELECTRON_MASS);
        if (kinetic_energy <= R(0.5) * m1 * m1 / R(ELECTRON_MASS))
            return analytic_ionisation_recoil_integral<R>(moment, kinetic_energy, xlow, el, mass);
    }
    return recoil_integral<R>(process, moment, kinetic_energy, xlow, el, mass, min_points);
}

} // namespace noa_oracle
