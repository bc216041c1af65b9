/*
 * Elastic (Coulomb) scattering per kinetic energy, FP64, one thread per K:
 *
 *   coulomb_data       dcs.hh:499-622  CM Lorentz factors, spin factor,
 *                                      screening parameters + pole factors,
 *                                      inverse Wentzel path
 *   coulomb_transport  dcs.hh:624-699  first two transport coefficients
 *                                      below a cut-off angle mu
 *   hard_scattering    dcs.hh:702-872  hard-scattering cut-off angle mu0 and
 *                                      mean free path lb_h over nel elements,
 *                                      by Ridders' method (numerics.hh:154-216)
 *
 * This translation unit is compiled with -fmad=false so that every product
 * and sum is rounded as in the reference (no FMA contraction); the Ridders
 * iteration branches on the signs of objective values, and a contracted
 * expression could change its path.  pow(A, 1/3), pow(Z, 2/3) and the
 * maximum hard angle are per-element constants computed once on the host
 * with the C library (the reference computes the same values per call).
 *
 * These are scalar, branchy, per-K computations (a few logs, a series of
 * 10 + Z terms, up to 100 root iterations): latency bound, a few microseconds
 * per million energies, far from any roofline that matters next to the DCS
 * kernels.  Records are the reference's: fCM [n][2], screen [n][9].
 */
#include "dcs_launch.h"

#include <cuda_runtime.h>

namespace noa_coulomb {

constexpr int NSF = 9;
constexpr double ATOMIC_MASS_ENERGY = 0.931494;  // physics.hh:55
constexpr double KIN_CUTOFF = 1E-9;              // physics.hh:78
constexpr double EHS_PATH_MAX = 1E+9;            // physics.hh:79
constexpr double EHS_OVER_MSC = 1E-4;            // physics.hh:80

// std::min's rule (b < a ? b : a), which differs from fmin for NaN.
__device__ __forceinline__ double smin(double a, double b) { return (b < a) ? b : a; }

__device__ __forceinline__ double frame_parameters(double *fCM, double K, const noa_coulomb_element &e, double mass) {
    const double Ma = e.A * ATOMIC_MASS_ENERGY;
    double M2 = mass + Ma;
    M2 *= M2;
    const double sCM12i = 1. / sqrt(M2 + 2. * Ma * K);
    fCM[0] = (K + mass + Ma) * sCM12i;
    double kinetic0 = (K * Ma + mass * (mass + Ma)) * sCM12i - mass;
    if (kinetic0 < KIN_CUTOFF)
        kinetic0 = KIN_CUTOFF;
    const double etot = K + mass + Ma;
    const double betaCM2 = K * (K + 2. * mass) / (etot * etot);
    double rM2 = mass / Ma;
    rM2 *= rM2;
    fCM[1] = sqrt(rM2 * (1. - betaCM2) + betaCM2);
    return kinetic0;
}

__device__ __forceinline__ double screening_parameters(double *ps, double K, const noa_coulomb_element &e,
                                                       double mass) {
    const double R1 = 1.02934 * e.A13 + 0.435;
    const double R2 = 2.;
    const double p2 = K * (K + 2. * mass);
    const double d = 5.8406E-02 / p2;
    ps[1] = d / (R1 * R1);
    ps[2] = d / (R2 * R2);

    // Moliere atomic screening with Kuraev's Coulomb correction, dcs.hh:560-590
    const int Z = e.Z;
    const double etot = K + mass;
    const double ZE = Z * etot;
    const double zeta2 = 5.3251346E-05 * (ZE * ZE) / p2;
    double cK;
    if (zeta2 > 1.) {
        const int n = 10 + Z;
        double f = 0.;
        for (int i = 1; i <= n; i++)
            f += zeta2 / (i * (i * i + zeta2));
        cK = exp(f);
    } else {
        cK = exp(1. - 1. / (1. + zeta2) + zeta2 * (0.2021 + zeta2 * (0.0083 * zeta2 - 0.0369)));
    }
    const double cM = 1. + 3.34 * zeta2;
    double r = K / etot;
    r *= r;
    const double c = r * cK + (1. - r) * cM;
    ps[0] = 5.179587126E-12 * e.Z23 * c / p2;

    // pole reduction factors, dcs.hh:592-599
    const double d01 = 1. / (ps[0] - ps[1]);
    const double d02 = 1. / (ps[0] - ps[2]);
    const double d12 = 1. / (ps[1] - ps[2]);
    ps[6] = d01 * d01 * d02 * d02;
    ps[7] = d01 * d01 * d12 * d12;
    ps[8] = d12 * d12 * d02 * d02;
    ps[3] = 2. * ps[6] * (d01 + d02);
    ps[4] = 2. * ps[7] * (d12 - d01);
    ps[5] = -2. * ps[8] * (d12 + d02);

    // inverse Wentzel path, dcs.hh:531-538
    const double dw = K * (K + 2. * mass) / (Z * (K + mass));
    return 1. / (e.A * 2.54910918E+08 * ps[0] * (1. + ps[0]) * dw * dw);
}

__global__ void __launch_bounds__(128) coulomb_data_kernel(const double *__restrict__ K, int64_t n,
                                                           const noa_coulomb_element e, double mass,
                                                           double *__restrict__ fCM, double *__restrict__ screen,
                                                           double *__restrict__ fspin,
                                                           double *__restrict__ invlambda) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double f[2], ps[NSF];
        const double kinetic0 = frame_parameters(f, K[i], e, mass);
        const double ek = kinetic0 + mass;  // spin factor, dcs.hh:525-528
        fspin[i] = kinetic0 * (ek + mass) / (ek * ek);
        invlambda[i] = screening_parameters(ps, kinetic0, e, mass);
        fCM[2 * i] = f[0];
        fCM[2 * i + 1] = f[1];
#pragma unroll
        for (int j = 0; j < NSF; j++)
            screen[NSF * i + j] = ps[j];
    }
}

// dcs.hh:624-677
__device__ __forceinline__ void transport_coefficients(double *coefs, const double *ps, double fspin, double mu) {
    const double nuclear_screening = (ps[1] < ps[2]) ? ps[1] : ps[2];
    if (mu < 1E-08 * nuclear_screening) {
        const double L = log(1. + mu / ps[0]);
        const double r = mu / (mu + ps[0]);
        const double k = ps[0] * (1. + ps[0]);
        coefs[0] = k * (r / ps[0] - fspin * (L - r));
        const double I2 = mu - ps[0] * (r - 2. * L);
        coefs[1] = 2. * k * (L - r - fspin * I2);
        return;
    }
    const double mu2 = 0.5 * mu * mu;
    double c0 = 0., c1 = 0.;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        double r = mu / (mu + ps[i]);
        double L = log(1. + mu / ps[i]);
        double mu1 = mu;
        const double I0 = r / ps[i];
        const double J0 = L;
        const double I1 = L - r;
        r *= ps[i];
        L *= ps[i];
        const double J1 = mu1 - L;
        const double I2 = mu1 - 2. * L + r;
        L *= ps[i];
        mu1 *= ps[i];
        const double J2 = mu2 + L - mu1;
        c0 += ps[3 + i] * (J0 - fspin * J1) + ps[6 + i] * (I0 - fspin * I1);
        c1 += ps[3 + i] * (J1 - fspin * J2) + ps[6 + i] * (I1 - fspin * I2);
    }
    const double k = ps[0] * (1. + ps[0]) * ps[1] * ps[1] * ps[2] * ps[2];
    coefs[0] = c0 * k;
    coefs[1] = c1 * (2. * k);
}

__global__ void __launch_bounds__(128) coulomb_transport_kernel(const double *__restrict__ screen,
                                                                const double *__restrict__ fspin,
                                                                const double *__restrict__ mu, int64_t n_mu,
                                                                int64_t n, double *__restrict__ coefs) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double ps[NSF], c[2];
#pragma unroll
        for (int j = 0; j < NSF; j++)
            ps[j] = screen[NSF * i + j];
        transport_coefficients(c, ps, fspin[i], mu[n_mu == 1 ? 0 : i]);
        coefs[2 * i] = c[0];
        coefs[2 * i + 1] = c[1];
    }
}

// dcs.hh:702-740
__device__ __forceinline__ double restricted_cs(double mu, double fspin, const double *__restrict__ s) {
    if (mu >= 1.)
        return 0.;
    const double nuclear_screening = (s[1] < s[2]) ? s[1] : s[2];
    if (mu < 1E-08 * nuclear_screening) {
        const double L = log((s[0] + 1.) / (s[0] + mu));
        const double r = (1. - mu) / ((s[0] + mu) * (s[0] + 1.));
        const double k = s[0] * (1. + s[0]);
        return k * (r - fspin * (L - s[0] * r));
    }
    double cs = 0.;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const double L = log((s[i] + 1.) / (s[i] + mu));
        const double r = (1. - mu) / ((s[i] + mu) * (s[i] + 1.));
        const double I0 = r, J0 = L, I1 = L - s[i] * r, J1 = mu - s[i] * L;
        cs += s[3 + i] * (J0 - fspin * J1) + s[6 + i] * (I0 - fspin * I1);
    }
    const double k = s[0] * (1. + s[0]) * s[1] * s[1] * s[2] * s[2];
    return k * cs;
}

struct HardArgs {
    const double *G, *fCM, *screen, *invlambda, *fspin;
    int64_t nel, nkin;
};

// dcs.hh:742-752 for energy index i.
__device__ __forceinline__ double objective(const HardArgs &a, int64_t i, double cs_h, double mu) {
    double cs_tot = 0.;
    for (int64_t iel = 0; iel < a.nel; iel++) {
        const int64_t off = iel * a.nkin + i;
        cs_tot += a.invlambda[off] * restricted_cs(mu, a.fspin[off], a.screen + NSF * off);
    }
    return cs_tot - cs_h;
}

// Ridders' method, numerics.hh:154-216; false where the reference returns
// an empty optional.
__device__ bool ridders(const HardArgs &a, int64_t i, double cs_h, double xa, double xb, double fa, double fb,
                        double xtol, double rtol, int max_iter, double &root) {
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
    const double tol = xtol + rtol * smin(fabs(xa), fabs(xb));
    for (int it = 0; it < max_iter; it++) {
        double dm = 0.5 * (xb - xa);
        const double xm = xa + dm;
        const double fm = objective(a, i, cs_h, xm);
        double sgn = (fb > fa) ? 1. : -1.;
        double dn = sgn * dm * fm / sqrt(fm * fm - fa * fb);
        sgn = (dn > 0.) ? 1. : -1.;
        dn = fabs(dn);
        dm = fabs(dm) - 0.5 * tol;
        if (dn < dm)
            dm = dn;
        const double xn = xm - sgn * dm;
        const double fn = objective(a, i, cs_h, xn);
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
        if (fn == 0.0 || fabs(xb - xa) < tol) {
            root = xn;
            return true;
        }
    }
    return false;
}

__global__ void __launch_bounds__(128) hard_scattering_kernel(const HardArgs a, double max_mu0,
                                                              double *__restrict__ mu0_out,
                                                              double *__restrict__ lb_h_out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.nkin;
         i += (int64_t)gridDim.x * blockDim.x) {
        double invlb_m = 0., invlb1_m = 0., s_m_l = 0., s_m_h = 0.;
        for (int64_t iel = 0; iel < a.nel; iel++) {
            const int64_t off = iel * a.nkin + i;
            const double invlb = a.invlambda[off];
            const double scr = a.screen[NSF * off];
            invlb_m += invlb * a.G[2 * off];
            s_m_h += scr * invlb;
            s_m_l += invlb / scr;
            const double d = 1. / (a.fCM[2 * off] * (1. + a.fCM[1 + 2 * off]));
            invlb1_m += invlb * a.G[1 + 2 * off] * d * d;
        }
        const double lb_m = 1. / invlb_m;
        double lb_h = smin(EHS_OVER_MSC / invlb1_m, EHS_PATH_MAX);
        double mu0;
        if (!(lb_m < lb_h)) {
            lb_h = lb_m;
            mu0 = 0;
        } else {
            const double s_m = (lb_h > 2. * lb_m) ? s_m_h * lb_m : 1. / (s_m_l * lb_m);
            mu0 = s_m * (lb_h - lb_m) / (s_m * lb_h + lb_m);
            const double cs_h = 1. / lb_h;
            double mu_max = smin(4. * mu0, 1.);
            double mu_min = 0.25 * mu0;
            double fmax = objective(a, i, cs_h, mu_max);
            // fmax > 0: the reference keeps the asymptotic mu0 and lb_h
            if (!(fmax > 0.)) {
                double fmin_ = objective(a, i, cs_h, mu_min);
                if (fmin_ < 0.) {
                    mu_max = mu_min;
                    fmax = fmin_;
                    mu_min = 0.;
                    fmin_ = objective(a, i, cs_h, mu_min);
                }
                if (mu_min < max_mu0) {
                    mu_max = smin(mu_max, max_mu0);
                    double root;
                    if (ridders(a, i, cs_h, mu_min, mu_max, fmin_, fmax, 1E-6 * mu0, 1E-6, 100, root))
                        mu0 = root;
                }
                mu0 = smin(mu0, max_mu0);
                lb_h = objective(a, i, cs_h, mu0) + cs_h;
                lb_h = (lb_h <= 1. / EHS_PATH_MAX) ? EHS_PATH_MAX : 1. / lb_h;
            }
        }
        mu0_out[i] = mu0;
        lb_h_out[i] = lb_h;
    }
}

int grid_for(int64_t n, int threads) {
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t blocks = (n + threads - 1) / threads;
    const int64_t cap = (int64_t)sms * 16;
    return (int)(blocks < cap ? blocks : cap);
}

} // namespace noa_coulomb

using namespace noa_coulomb;

cudaError_t noa_dcs_launch_coulomb_data(const double *K, int64_t n, const noa_coulomb_element *e, double mass,
                                        double *fCM, double *screen, double *fspin, double *invlambda,
                                        cudaStream_t stream) {
    if (n <= 0)
        return cudaSuccess;
    coulomb_data_kernel<<<grid_for(n, 128), 128, 0, stream>>>(K, n, *e, mass, fCM, screen, fspin, invlambda);
    return cudaGetLastError();
}

cudaError_t noa_dcs_launch_coulomb_transport(const double *screen, const double *fspin, const double *mu,
                                             int64_t n_mu, int64_t n, double *coefs, cudaStream_t stream) {
    if (n <= 0)
        return cudaSuccess;
    coulomb_transport_kernel<<<grid_for(n, 128), 128, 0, stream>>>(screen, fspin, mu, n_mu, n, coefs);
    return cudaGetLastError();
}

cudaError_t noa_dcs_launch_hard_scattering(const double *G, const double *fCM, const double *screen,
                                           const double *invlambda, const double *fspin, int64_t nel, int64_t nkin,
                                           double max_mu0, double *mu0, double *lb_h, cudaStream_t stream) {
    if (nkin <= 0)
        return cudaSuccess;
    HardArgs a{G, fCM, screen, invlambda, fspin, nel, nkin};
    hard_scattering_kernel<<<grid_for(nkin, 128), 128, 0, stream>>>(a, max_mu0, mu0, lb_h);
    return cudaGetLastError();
}
