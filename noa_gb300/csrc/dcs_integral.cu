/*
 * Recoil-energy integrals of the DCS per kinetic energy (FP64):
 *
 *   DEL: (1/E) int_{K xlow}^{K} q dsigma/dq dq      (moment 0)
 *   CEL: (1/E) int_{K xlow}^{K} q^2 dsigma/dq dq    (moment 1)
 *
 * Reference: recoil_integral (src/noa/pms/dcs.hh:89-105) with del_integrand /
 * cel_integrand (:107-113), mapped by vmap_integral (:115-130): a composite
 * 6-node Gauss-Legendre rule (numerics.hh:71-108) over t = log q with
 * n_itv = ceil(min_points / 6) intervals, i.e. 6 n_itv DCS evaluations per
 * K; ionisation switches to its closed form below the radiative-correction
 * threshold (dcs.hh:446-496, 955-1001).
 *
 * Kernel: a CTA takes a tile of kpt kinetic energies and all their nodes
 * (kpt * nodes pairs, at most 1536).  Each pair (K, q_i) is classified with the
 * process's exact bounds; closed pairs contribute 0, open ones go to the
 * shared-memory work queue and are evaluated 256 at a time with every lane
 * busy.  Each weighted node value lands in a shared array indexed by
 * (K, node), and one thread per K then sums its nodes in node order -- the
 * reference's own order -- so the result does not depend on scheduling.
 */
#include "dcs_fp64.cuh"
#include "dcs_launch.h"

#include <cuda_runtime.h>

namespace noa_dcs {

constexpr int I_THREADS = 256;
constexpr int I_PAIRS = 1536;  // pairs per tile (kpt * nodes <= I_PAIRS)
constexpr int I_QCAP = I_PAIRS + I_THREADS;
constexpr int I_KMAX = 128;    // kinetic energies per tile at most

__constant__ double kGL6X[6] = {0.03376524, 0.16939531, 0.38069041, 0.61930959, 0.83060469, 0.96623476};
__constant__ double kGL6W[6] = {0.08566225, 0.18038079, 0.23395697, 0.23395697, 0.18038079, 0.08566225};

struct IntegralParams {
    const double *K;
    double *out;
    int64_t n;
    double xlow;
    int nodes;  // 6 * n_itv
    int n_itv;
    int kpt;    // kinetic energies per tile
    int moment; // 0 = DEL, 1 = CEL
};

template <int PROC>
__device__ __forceinline__ double i_eval(double K, double q, const noa_dcs_consts &c) {
    if (PROC == NOA_DCS_PROC_BREMS)
        return brems_fp64(K, q, c);
    else if (PROC == NOA_DCS_PROC_PPROD)
        return pprod_fp64(K, q, c);
    else if (PROC == NOA_DCS_PROC_PHOTO)
        return photo_fp64(K, q, c);
    else
        return ion_fp64(K, q, c);
}

template <int PROC>
__device__ __forceinline__ bool i_open(double K, double q, const noa_dcs_consts &c) {
    if (PROC == NOA_DCS_PROC_PPROD)
        return pprod_live(K, q, c);
    else if (PROC == NOA_DCS_PROC_PHOTO)
        return photo_live(K, q, c);
    else if (PROC == NOA_DCS_PROC_ION) {
        // ionisation's early returns, dcs.hh:415-424
        const double P2 = K * (K + 2. * c.mass);
        const double Wmax = ion_wmax(P2, K + c.mass, c);
        return !((Wmax < NOA_X_FRACTION * K) || (q > Wmax) || (q <= c.io_Wmin));
    } else
        return true;
}

// The closed-form ionisation integrals, dcs.hh:446-496 (FP64, IEEE order).
__device__ __forceinline__ double ion_analytic(double K, double xlow, int moment, const noa_dcs_consts &c) {
    const double mass = c.mass;
    const double P2 = K * (K + 2. * mass);
    const double E = K + mass;
    const double Wmax = ion_wmax(P2, E, c);
    if (Wmax < NOA_X_FRACTION * K)
        return 0.;
    double Wmin = c.io_Wmin;
    const double qlow = K * xlow;
    if (qlow >= Wmin)
        Wmin = qlow;
    if (Wmax <= Wmin)
        return 0.;
    const double a0 = x_div(0.5, P2), a1 = x_div(-1., Wmax), a2 = x_div(E * E, P2);
    const double lw = log(x_div(Wmax, Wmin));
    double term;
    if (moment == 0)
        term = x_add(x_add(x_mul(a0, Wmax - Wmin), x_mul(a1, lw)), x_mul(a2, x_sub(x_div(1., Wmin), x_div(1., Wmax))));
    else
        term = x_add(x_add(x_mul(x_mul(0.5, a0), x_sub(x_mul(Wmax, Wmax), x_mul(Wmin, Wmin))), x_mul(a1, Wmax - Wmin)),
                     x_mul(a2, lw));
    return x_mul(x_div(x_mul(1.535336E-05, c.Zd), c.A), term);
}

__device__ __forceinline__ int i_scan(int v, int *warp_tot, int *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o)
            x += y;
    }
    if (lane == 31)
        warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
        const int w = lane < (I_THREADS >> 5) ? warp_tot[lane] : 0;
        int s = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o)
                s += y;
        }
        if (lane < (I_THREADS >> 5))
            warp_tot[lane] = s - w;
        if (lane == 31)
            *total = s;
    }
    __syncthreads();
    return warp_tot[warp] + x - v;
}

// Weighted value of node slot (f h w of numerics.hh:86, f = dcs q or dcs q^2).
template <int PROC>
__device__ __forceinline__ double i_node_value(double K, double q, double h, int node, int moment,
                                               const noa_dcs_consts &c) {
    const double d = i_eval<PROC>(K, q, c);
    const double f = moment == 0 ? x_mul(d, q) : x_mul(x_mul(d, q), q);
    return x_mul(x_mul(f, h), kGL6W[node % 6]);
}

template <int PROC>
__global__ void __launch_bounds__(I_THREADS) recoil_integral_kernel(const IntegralParams p, const noa_dcs_consts c) {
    __shared__ double vals[I_PAIRS];   // weighted node values of the tile, [k][node]
    __shared__ double qQ[I_QCAP];      // queued recoil energies
    __shared__ int qS[I_QCAP];         // their slots in vals
    __shared__ double sK[I_KMAX], sLb[I_KMAX], sH[I_KMAX];
    __shared__ int warp_tot[I_THREADS / 32];
    __shared__ int tile_open;
    const int pairs = p.kpt * p.nodes;
    const int64_t tiles = (p.n + p.kpt - 1) / p.kpt;
    const double ion_thr = c.io_k_rad;  // 0.5 (m - me)^2 / me, dcs.hh:962-963

    for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const int64_t k0 = tile * p.kpt;
        if ((int)threadIdx.x < p.kpt) {
            // bounds of the t = log q rule for this K, numerics.hh:80-81
            const int64_t ki = k0 + threadIdx.x;
            const double K = ki < p.n ? p.K[ki] : 1.;
            const double lb = log(K * p.xlow), ub = log(K);
            sK[threadIdx.x] = K;
            sLb[threadIdx.x] = lb;
            sH[threadIdx.x] = x_div(ub - lb, fpconv::f64i(p.n_itv));
        }
        __syncthreads();
        int qn = 0;
        for (int base = 0;; base += I_THREADS) {
            const bool more = base < pairs;  // block-uniform
            if (more) {
                const int slot = base + threadIdx.x;
                bool open = false;
                double q = 0.;
                if (slot < pairs) {
                    const int kk = slot / p.nodes, i = slot - kk * p.nodes;
                    vals[slot] = 0.;
                    const double K = sK[kk];
                    if (k0 + kk < p.n && !(PROC == NOA_DCS_PROC_ION && K <= ion_thr)) {
                        // node i of the composite rule, numerics.hh:84-86, in IEEE order
                        const double t = x_add(sLb[kk], x_mul(sH[kk], fpconv::f64i(i / 6) + kGL6X[i % 6]));
                        q = lean_exp(t);
                        open = i_open<PROC>(K, q, c);
                    }
                }
                const int pos = qn + i_scan(open ? 1 : 0, warp_tot, &tile_open);
                if (open) {
                    qQ[pos] = q;
                    qS[pos] = slot;
                }
                __syncthreads();
                qn += tile_open;
            }
            // one call site of the evaluation (a pair's rounding must not
            // depend on its queue position): full batches, then the rest
            while (qn >= I_THREADS || (!more && qn > 0)) {
                const int take = qn < I_THREADS ? qn : I_THREADS;
                if ((int)threadIdx.x < take) {
                    const int e = qn - take + threadIdx.x;
                    const int sl = qS[e], kk = sl / p.nodes;
                    vals[sl] = i_node_value<PROC>(sK[kk], qQ[e], sH[kk], sl - kk * p.nodes, p.moment, c);
                }
                qn -= take;
                __syncthreads();
            }
            if (!more)
                break;
        }
        // one thread per kinetic energy: node-ordered sum, as the reference
        if ((int)threadIdx.x < p.kpt) {
            const int64_t ki = k0 + threadIdx.x;
            if (ki < p.n) {
                const double K = sK[threadIdx.x];
                double r;
                if (PROC == NOA_DCS_PROC_ION && K <= ion_thr) {
                    r = ion_analytic(K, p.xlow, p.moment, c);
                } else {
                    double s = 0.;
                    const double *v = vals + threadIdx.x * p.nodes;
                    for (int i = 0; i < p.nodes; i++)
                        s = x_add(s, v[i]);
                    r = x_div(s, K + c.mass);
                }
                p.out[ki] = r;
            }
        }
        __syncthreads();
    }
}

// ------------------------------------------------ soft-scattering transport
/*
 * soft_scattering (dcs.hh:941-952) per K: the closed-form ionisation part
 * (dcs.hh:874-899) plus twice a 6-node composite GL rule over
 * t = log(nu / X_FRACTION) on [log 1e-6, 0] with 17 intervals (102 nodes) of
 * photonuclear(K, q) * ratio(K, q) * nu, q = nu K, where ratio is the
 * mu-integrated angular weight of dcs.hh:911-934.  Same tile / queue scheme
 * as the recoil integrals: closed photonuclear nodes contribute
 * 0 * ratio * nu (0, or NaN where the weight is not finite, as in the
 * reference), open ones are evaluated 256 at a time.
 */
constexpr int S_NODES = 102;            // 6 * ceil(100 / 6)
constexpr int S_KPT = I_PAIRS / S_NODES; // 15 kinetic energies per tile
constexpr int S_PAIRS = S_KPT * S_NODES;

struct SoftParams {
    const double *K;
    double *out;
    int64_t n;
    double lb;  // log(1e-6)
    double h;   // -lb / 17
};

// dcs.hh:913-934 in the reference's operation order.
__device__ __forceinline__ double soft_ratio(double K, double q, double mass) {
    const double E = x_add(K, mass);
    const double m02 = 0.4;
    const double q2 = x_mul(q, q);
    const double tmax = x_mul(1.876544, q);
    const double tmin = x_div(x_mul(x_mul(q2, mass), mass), x_mul(E, x_sub(E, q)));
    const double b1 = x_div(1., x_sub(1., x_div(q2, m02)));
    const double c1 = x_div(1., x_sub(1., x_div(m02, q2)));
    double L1 = x_mul(b1, log(x_div(x_add(q2, tmax), x_add(q2, tmin))));
    double L2 = x_mul(c1, log(x_div(x_add(m02, tmax), x_add(m02, tmin))));
    const double I0 = x_sub(x_sub(log(x_div(tmax, tmin)), L1), L2);
    L1 = x_mul(L1, q2);
    L2 = x_mul(L2, m02);
    const double I1 = x_add(L1, L2);
    L1 = x_mul(L1, q2);
    L2 = x_mul(L2, m02);
    const double I2 = x_sub(x_sub(x_mul(x_sub(tmax, tmin), x_add(x_mul(b1, q2), x_mul(c1, m02))), L1), L2);
    return x_div(x_sub(x_mul(I1, tmax), I2),
                 x_mul(x_mul(x_sub(x_mul(I0, tmax), I1), K), x_add(K, x_mul(2., mass))));
}

// The same weight with the lean functions, for closed photonuclear nodes:
// there the reference adds 0 * ratio * nu, which is 0 (of either sign, which
// the node sum cannot tell apart) unless the ratio is not finite.  Only its
// finiteness is used.
__device__ __forceinline__ bool soft_ratio_finite(double K, double q, double mass) {
    const double E = K + mass;
    const double m02 = 0.4;
    const double q2 = x_mul(q, q);
    const double tmax = 1.876544 * q;
    const double tmin = q2 * mass * mass * d_rcp(E * (E - q));
    // the weight's poles (q^2 = m02) are decided in IEEE arithmetic as in the reference
    const double b1 = d_rcp(x_sub(1., x_div(q2, m02)));
    const double c1 = d_rcp(x_sub(1., x_div(m02, q2)));
    double L1 = b1 * d_log((q2 + tmax) * d_rcp(q2 + tmin));
    double L2 = c1 * d_log((m02 + tmax) * d_rcp(m02 + tmin));
    const double I0 = d_log(tmax * d_rcp(tmin)) - L1 - L2;
    L1 *= q2;
    L2 *= m02;
    const double I1 = L1 + L2;
    L1 *= q2;
    L2 *= m02;
    const double I2 = (tmax - tmin) * (b1 * q2 + c1 * m02) - L1 - L2;
    const double r = (I1 * tmax - I2) * d_rcp((I0 * tmax - I1) * K * (K + 2. * mass));
    return isfinite(r);
}

// dcs.hh:874-899 in the reference's operation order.
__device__ __forceinline__ double soft_ionisation(double K, const noa_dcs_consts &c) {
    const double mass = c.mass;
    const double p2 = x_mul(K, x_add(K, x_mul(2., mass)));
    const double E = x_add(K, mass);
    const double Wmax = x_div(x_mul(x_mul(2., ME), p2), x_add(x_mul(mass, mass), x_mul(ME, x_add(ME, x_mul(2., E)))));
    const double W0 = x_div(x_mul(2., p2), ME);
    const double mu_max = x_div(Wmax, W0);
    double mu3 = x_div(x_mul(K, NOA_X_FRACTION), W0);
    if (mu3 > mu_max)
        mu3 = mu_max;
    const double mu2 = x_div(x_mul(0.62, c.I), W0);
    if (mu2 >= mu3)
        return 0.;
    const double a0 = x_div(x_mul(0.5, W0), p2);
    const double a1 = x_div(-1., Wmax);
    const double a2 = x_div(x_mul(E, E), x_mul(W0, p2));
    const double cs0 = x_div(1.535336E-05, c.A);
    const double bracket = x_add(x_add(x_mul(x_mul(0.5, a0), x_sub(x_mul(mu3, mu3), x_mul(mu2, mu2))),
                                       x_mul(a1, x_sub(mu3, mu2))),
                                 x_mul(a2, log(x_div(mu3, mu2))));
    return x_mul(x_mul(x_mul(2., cs0), c.Zd), bracket);
}

// Node i of the rule for kinetic energy K: nu and q (numerics.hh:84-86, dcs.hh:910-911).
__device__ __forceinline__ void soft_node(double K, int i, const SoftParams &p, double &nu, double &q) {
    const double t = x_add(p.lb, x_mul(p.h, fpconv::f64i(i / 6) + kGL6X[i % 6]));
    nu = x_mul(NOA_X_FRACTION, exp(t));
    q = x_mul(nu, K);
}

__global__ void __launch_bounds__(I_THREADS) soft_scattering_kernel(const SoftParams p, const noa_dcs_consts c) {
    __shared__ double vals[S_PAIRS];
    __shared__ int qS[S_PAIRS + I_THREADS];
    __shared__ double sK[S_KPT];
    __shared__ int warp_tot[I_THREADS / 32];
    __shared__ int tile_open;
    const int64_t tiles = (p.n + S_KPT - 1) / S_KPT;

    for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const int64_t k0 = tile * S_KPT;
        if ((int)threadIdx.x < S_KPT) {
            const int64_t ki = k0 + threadIdx.x;
            sK[threadIdx.x] = ki < p.n ? p.K[ki] : 1.;
        }
        __syncthreads();
        int qn = 0;
        for (int base = 0;; base += I_THREADS) {
            const bool more = base < S_PAIRS;  // block-uniform
            if (more) {
                const int slot = base + threadIdx.x;
                bool open = false;
                if (slot < S_PAIRS) {
                    const int kk = slot / S_NODES, i = slot - kk * S_NODES;
                    vals[slot] = 0.;
                    if (k0 + kk < p.n) {
                        const double K = sK[kk];
                        double nu, q;
                        soft_node(K, i, p, nu, q);
                        open = photo_live(K, q, c);
                        if (!open && !soft_ratio_finite(K, q, c.mass))  // photonuclear = 0: 0 * ratio * nu
                            vals[slot] = __longlong_as_double(0x7FF8000000000000LL);   // NaN, as 0 * inf
                    }
                }
                const int pos = qn + i_scan(open ? 1 : 0, warp_tot, &tile_open);
                if (open)
                    qS[pos] = slot;
                __syncthreads();
                qn += tile_open;
            }
            // one call site of the evaluation, as in the recoil integrals
            while (qn >= I_THREADS || (!more && qn > 0)) {
                const int take = qn < I_THREADS ? qn : I_THREADS;
                if ((int)threadIdx.x < take) {
                    const int sl = qS[qn - take + threadIdx.x];
                    const int kk = sl / S_NODES, i = sl - kk * S_NODES;
                    const double K = sK[kk];
                    double nu, q;
                    soft_node(K, i, p, nu, q);
                    const double f = x_mul(x_mul(photo_fp64(K, q, c), soft_ratio(K, q, c.mass)), nu);
                    vals[sl] = x_mul(x_mul(f, p.h), kGL6W[i % 6]);
                }
                qn -= take;
                __syncthreads();
            }
            if (!more)
                break;
        }
        __syncthreads();
        if ((int)threadIdx.x < S_KPT) {
            const int64_t ki = k0 + threadIdx.x;
            if (ki < p.n) {
                double s = 0.;
                const double *v = vals + threadIdx.x * S_NODES;
                for (int i = 0; i < S_NODES; i++)
                    s = x_add(s, v[i]);
                p.out[ki] = x_add(soft_ionisation(sK[threadIdx.x], c), x_mul(2., s));
            }
        }
        __syncthreads();
    }
}

static int sm_count() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

} // namespace noa_dcs

using namespace noa_dcs;

cudaError_t noa_dcs_launch_recoil_integral(int process, int moment, const double *K, double *out, int64_t n,
                                           double xlow, int min_points, const noa_dcs_consts *c,
                                           cudaStream_t stream) {
    if (n <= 0)
        return cudaSuccess;
    IntegralParams p;
    p.K = K;
    p.out = out;
    p.n = n;
    p.xlow = xlow;
    p.n_itv = (min_points + 5) / 6;
    p.nodes = 6 * p.n_itv;
    if (p.nodes > I_PAIRS || p.nodes < 6)
        return cudaErrorInvalidValue;
    p.kpt = I_PAIRS / p.nodes;
    if (p.kpt > I_KMAX)
        p.kpt = I_KMAX;
    p.moment = moment;
    const int64_t tiles = (n + p.kpt - 1) / p.kpt;
    const int64_t cap = (int64_t)sm_count() * 3;
    const int grid = (int)(tiles < cap ? tiles : cap);
    switch (process) {
    case NOA_DCS_PROC_BREMS:
        recoil_integral_kernel<NOA_DCS_PROC_BREMS><<<grid, I_THREADS, 0, stream>>>(p, *c);
        break;
    case NOA_DCS_PROC_PPROD:
        recoil_integral_kernel<NOA_DCS_PROC_PPROD><<<grid, I_THREADS, 0, stream>>>(p, *c);
        break;
    case NOA_DCS_PROC_PHOTO:
        recoil_integral_kernel<NOA_DCS_PROC_PHOTO><<<grid, I_THREADS, 0, stream>>>(p, *c);
        break;
    case NOA_DCS_PROC_ION:
        recoil_integral_kernel<NOA_DCS_PROC_ION><<<grid, I_THREADS, 0, stream>>>(p, *c);
        break;
    default:
        return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t noa_dcs_launch_soft_scattering(const double *K, double *out, int64_t n, const noa_dcs_consts *c,
                                           cudaStream_t stream) {
    if (n <= 0)
        return cudaSuccess;
    SoftParams p;
    p.K = K;
    p.out = out;
    p.n = n;
    p.lb = log(1E-06);                // dcs.hh:905
    p.h = (0. - p.lb) / (double)17u;  // numerics.hh:80-81, n_itv = ceil(100 / 6)
    const int64_t tiles = (n + S_KPT - 1) / S_KPT;
    const int64_t cap = (int64_t)sm_count() * 3;
    const int grid = (int)(tiles < cap ? tiles : cap);
    soft_scattering_kernel<<<grid, I_THREADS, 0, stream>>>(p, *c);
    return cudaGetLastError();
}
