/*
 * C entry points of the CPU oracle -- TEST INFRASTRUCTURE ONLY.
 *
 * Serial and OpenMP element maps over the restated DCS functions of
 * dcs_oracle.hpp, mirroring the reference's dcs::vmap (dcs.hh:35-48, a serial
 * loop, common.hh:146-152) and dcs::pvmap (dcs.hh:62-75, an OpenMP static
 * parallel for, common.hh:154-161), the per-K recoil integrals
 * (vmap_integral, dcs.hh:115-130) and an operation counter that yields the
 * algorithmic flop-equivalents per evaluation.
 *
 * Built into oracle/liboracle_dcs.so by oracle/build_oracle.py; loaded by the
 * tests and by the CPU baseline of bench.py through ctypes.  The product
 * library never links it.
 */
#include "coulomb_oracle.hpp"
#include "dcs_oracle.hpp"

#include <omp.h>

#include <cstdint>
#include <cstring>

using namespace noa_oracle;

extern "C" {

/* Evaluates one process over n (K, q) pairs into out.  threads <= 0 uses
 * every OpenMP thread, 1 runs the serial loop (dcs::vmap), more runs the
 * OpenMP static loop (dcs::pvmap) on that many threads.  Returns 0, or -1 for
 * an unknown process. */
int oracle_dcs_vmap(int process, const double *K, const double *q, double *out, int64_t n, double A, double I,
                    int32_t Z, double mass, int threads) {
    if (process < 0 || process > 3)
        return -1;
    const Element el{A, I, Z};
    if (threads == 1) {
        for (int64_t i = 0; i < n; i++)
            out[i] = dcs<double>(process, K[i], q[i], el, mass);
        return 0;
    }
    const int nt = threads <= 0 ? omp_get_max_threads() : threads;
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int64_t i = 0; i < n; i++)
        out[i] = dcs<double>(process, K[i], q[i], el, mass);
    return 0;
}

/* Per-K recoil integral: moment 0 = DEL (int dcs*q), 1 = CEL (int dcs*q^2)
 * over q in [K*xlow, K], with the ionisation closed form below its
 * radiative-correction threshold (dcs.hh:955-1001).  Same threading rule as
 * oracle_dcs_vmap. */
int oracle_recoil_integral_vmap(int process, int moment, const double *K, double *out, int64_t n, double xlow,
                                double A, double I, int32_t Z, double mass, uint32_t min_points, int threads) {
    if (process < 0 || process > 3 || moment < 0 || moment > 1)
        return -1;
    const Element el{A, I, Z};
    const int nt = threads <= 0 ? omp_get_max_threads() : threads;
#pragma omp parallel for schedule(static) num_threads(nt) if (threads != 1)
    for (int64_t i = 0; i < n; i++)
        out[i] = recoil_integral_dispatch<double>(process, moment, K[i], xlow, el, mass, min_points);
    return 0;
}

int oracle_max_threads(void) { return omp_get_max_threads(); }

/* Elastic scattering per kinetic energy (coulomb_data, dcs.hh:604-622):
 * fCM [n][2], screen [n][9], fspin [n], invlambda [n]. */
int oracle_coulomb_data(const double *K, int64_t n, double A, double I, int32_t Z, double mass, double *fCM,
                        double *screen, double *fspin, double *invlambda) {
    const Element el{A, I, Z};
    for (int64_t i = 0; i < n; i++)
        coulomb_data(fCM + 2 * i, screen + NSF * i, fspin + i, invlambda + i, K[i], el, mass);
    return 0;
}

/* Transport coefficients (coulomb_transport, dcs.hh:679-699): coefs [n][2];
 * mu holds n_mu = 1 (shared) or n values. */
int oracle_coulomb_transport(const double *screen, const double *fspin, const double *mu, int64_t n_mu, int64_t n,
                             double *coefs) {
    for (int64_t i = 0; i < n; i++)
        coulomb_transport_coefficients(coefs + 2 * i, screen + NSF * i, fspin[i], mu[n_mu == 1 ? 0 : i]);
    return 0;
}

/* Hard-scattering cut-off and path (hard_scattering, dcs.hh:840-872) over
 * nel elements x nkin energies: G, fCM [nel][nkin][2], screen
 * [nel][nkin][9], invlambda, fspin [nel][nkin]; mu0, lb_h [nkin]. */
int oracle_hard_scattering(const double *G, const double *fCM, const double *screen, const double *invlambda,
                           const double *fspin, int64_t nel, int64_t nkin, double *mu0, double *lb_h) {
    for (int64_t i = 0; i < nkin; i++)
        coulomb_hard_scattering(mu0[i], lb_h[i], G + 2 * i, fCM + 2 * i, screen + NSF * i, invlambda + i,
                                fspin + i, nel, nkin);
    return 0;
}

/* Soft-scattering transverse transport per kinetic energy (soft_scattering,
 * dcs.hh:941-952).  Same threading rule as oracle_dcs_vmap. */
int oracle_soft_scattering(const double *K, double *out, int64_t n, double A, double I, int32_t Z, double mass,
                           int threads) {
    const Element el{A, I, Z};
    const int nt = threads <= 0 ? omp_get_max_threads() : threads;
#pragma omp parallel for schedule(static) num_threads(nt) if (threads != 1)
    for (int64_t i = 0; i < n; i++)
        out[i] = soft_scattering(K[i], el, mass);
    return 0;
}


/* Operation counts, accumulated over the n pairs by oracle_dcs_opcount.
 * Exported in this layout: add, mul, div, sqrt, cmp, transcendental. */
struct OpCounts {
    double add, mul, div, sqrt, cmp, trans;
};
}

namespace {

thread_local OpCounts g_ops;

/* A double that counts every arithmetic operation done on it.  Comparisons
 * count as one flop each, as do +, -, *, /, and sqrt; log, exp, pow and
 * log10 count once in `trans` (20 flop-equivalents each by convention). */
struct Cnt {
    double v;
    Cnt() : v(0) {}
    explicit Cnt(double x) : v(x) {}
};
inline Cnt operator+(Cnt a, Cnt b) { g_ops.add++; return Cnt(a.v + b.v); }
inline Cnt operator-(Cnt a, Cnt b) { g_ops.add++; return Cnt(a.v - b.v); }
inline Cnt operator-(Cnt a) { return Cnt(-a.v); }
inline Cnt operator*(Cnt a, Cnt b) { g_ops.mul++; return Cnt(a.v * b.v); }
inline Cnt operator/(Cnt a, Cnt b) { g_ops.div++; return Cnt(a.v / b.v); }
inline Cnt &operator+=(Cnt &a, Cnt b) { a = a + b; return a; }
inline Cnt &operator/=(Cnt &a, Cnt b) { a = a / b; return a; }
inline bool operator<(Cnt a, Cnt b) { g_ops.cmp++; return a.v < b.v; }
inline bool operator<=(Cnt a, Cnt b) { g_ops.cmp++; return a.v <= b.v; }
inline bool operator>(Cnt a, Cnt b) { g_ops.cmp++; return a.v > b.v; }
inline bool operator>=(Cnt a, Cnt b) { g_ops.cmp++; return a.v >= b.v; }
// Found by argument-dependent lookup from the templated oracle.
inline Cnt log(Cnt a) { g_ops.trans++; return Cnt(::log(a.v)); }
inline Cnt log10(Cnt a) { g_ops.trans++; return Cnt(::log10(a.v)); }
inline Cnt exp(Cnt a) { g_ops.trans++; return Cnt(::exp(a.v)); }
inline Cnt pow(Cnt a, Cnt b) { g_ops.trans++; return Cnt(::pow(a.v, b.v)); }
inline Cnt sqrt(Cnt a) { g_ops.sqrt++; return Cnt(::sqrt(a.v)); }
} // namespace

extern "C" {

/* Counts the operations of one process over n pairs (serially) and writes
 * the totals to counts[6] in the OpCounts order; also returns the checksum of
 * the counted evaluation (must equal the plain oracle's values). */
double oracle_dcs_opcount(int process, const double *K, const double *q, int64_t n, double A, double I, int32_t Z,
                          double mass, double *counts) {
    const Element el{A, I, Z};
    g_ops = OpCounts{0, 0, 0, 0, 0, 0};
    double checksum = 0;
    for (int64_t i = 0; i < n; i++)
        checksum += dcs<Cnt>(process, Cnt(K[i]), Cnt(q[i]), el, mass).v;
    std::memcpy(counts, &g_ops, sizeof(OpCounts));
    return checksum;
}
}
