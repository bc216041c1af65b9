/*
 * FP32-compensated DCS kernels (precision NOA_DCS_FP32C) for sm_103a.
 *
 * One kernel shape for all four processes, built on the compacting kernel of
 * the FP64 path (dcs_fp64.cu) with a second queue:
 *
 *   1. a CTA classifies a 1024-pair tile with the exact kinematic bounds
 *      (pair production, photonuclear; bremsstrahlung and ionisation are
 *      evaluated for every pair), writes the zeros, and appends the open
 *      pairs to the shared-memory work queue;
 *   2. whenever the work queue holds 256 pairs, each thread pops one and
 *      evaluates it in FP32 (dcs_fp32c.cuh), which also returns an estimate
 *      of its relative error; results within `tol` are written, the others
 *      are appended (warp-aggregated) to a shared-memory redo queue;
 *   3. whenever the redo queue holds 256 pairs, each thread pops one and
 *      evaluates it in FP64 (dcs_fp64.cuh) -- except for pair production,
 *      whose redo pairs are evaluated again in FP32 with the screening log in
 *      float-float arithmetic (pprod_fp32c<false, true>); the ~1% of those
 *      still above `tol` go to a third queue, evaluated in FP64 in batches of
 *      256 the same way.
 *
 * FP64 work is thus proportional to the redo fraction (0-0.5% of open pairs
 * at tol = 1e-6), and every warp of every phase runs with all lanes busy.
 * No global scratch.
 */
#include "dcs_fp32c.cuh"
#include "dcs_fp64.cuh"
#include "dcs_launch.h"

#include <cuda_runtime.h>

namespace noa_dcs {

constexpr int F_THREADS = 256;
constexpr int F_ITEMS = 4;
constexpr int F_TILE = F_THREADS * F_ITEMS;
constexpr int F_QCAP = F_TILE + F_THREADS;
constexpr int F_RCAP = 2 * F_THREADS;

// Resident CTAs per SM that each kernel is compiled for (its register budget
// follows).  Measured on 1e8 pairs: pair production is fastest at 2 (12.1 ms;
// 13.8 ms at 3, where it spills); photonuclear at 4 (4.32 ms against 4.60 ms
// at 3), with its FP64 redo out of line; the short bodies fit 4.
template <int PROC>
constexpr int f32_min_ctas() {
    return PROC == NOA_DCS_PROC_PPROD ? 2 : 4;
}

template <int PROC>
__device__ __forceinline__ double eval32(double K, double q, const noa_dcs_consts &c, float &est) {
    if (PROC == NOA_DCS_PROC_BREMS)
        return brems_fp32c(K, q, c, est);
    else if (PROC == NOA_DCS_PROC_PPROD)
        return pprod_fp32c<false>(K, q, c, est);
    else if (PROC == NOA_DCS_PROC_PHOTO)
        return photo_fp32c<false>(K, q, c, est);
    else
        return ion_fp32c(K, q, c, est);
}

template <int PROC>
__device__ __forceinline__ double eval64(double K, double q, const noa_dcs_consts &c) {
    if (PROC == NOA_DCS_PROC_BREMS)
        return brems_fp64(K, q, c);
    else if (PROC == NOA_DCS_PROC_PPROD)
        return pprod_fp64(K, q, c);
    else if (PROC == NOA_DCS_PROC_PHOTO)
        return photo_fp64(K, q, c);
    else
        return ion_fp64(K, q, c);
}

// The FP64 redo: out of line for the two quadrature processes
// (pprod_fp64_ol, photo_fp64_ol).
template <int PROC>
__device__ __forceinline__ double redo64(double K, double q, const noa_dcs_consts &c) {
    if (PROC == NOA_DCS_PROC_PPROD)
        return pprod_fp64_ol(K, q, c);
    else if (PROC == NOA_DCS_PROC_PHOTO)
        return photo_fp64_ol(K, q, c);
    return eval64<PROC>(K, q, c);
}

template <int PROC>
__device__ __forceinline__ bool open32(double K, double q, const noa_dcs_consts &c) {
    if (PROC == NOA_DCS_PROC_PPROD)
        return pprod_live(K, q, c);
    else if (PROC == NOA_DCS_PROC_PHOTO)
        return photo_live(K, q, c);
    else
        return true;
}

__device__ __forceinline__ int scan_block(int v, int *warp_tot, int *total) {
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
        const int w = lane < (F_THREADS >> 5) ? warp_tot[lane] : 0;
        int s = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o)
                s += y;
        }
        if (lane < (F_THREADS >> 5))
            warp_tot[lane] = s - w;
        if (lane == 31)
            *total = s;
    }
    __syncthreads();
    return warp_tot[warp] + x - v;
}

// The third queue exists for pair production only.
template <int PROC>
constexpr int f32_xcap() {
    return PROC == NOA_DCS_PROC_PPROD ? F_RCAP : 1;
}

template <int PROC>
struct Queues {
    double wK[F_QCAP], wQ[F_QCAP];
    int64_t wI[F_QCAP];
    double rK[F_RCAP], rQ[F_RCAP];
    int64_t rI[F_RCAP];
    double xK[f32_xcap<PROC>()], xQ[f32_xcap<PROC>()];
    int64_t xI[f32_xcap<PROC>()];
    int warp_tot[F_THREADS / 32];
    int tile_open;
    int rn, xn;
};

// Appends (k, q, i) of the lanes with `push` to a queue (warp-aggregated).
__device__ __forceinline__ void push_queue(bool push, double k, double q, int64_t i, double *QK, double *QQ,
                                           int64_t *QI, int *qn) {
    const unsigned m = __ballot_sync(0xffffffffu, push);
    if (m) {
        const int lane = threadIdx.x & 31;
        int base = 0;
        if (lane == 0)
            base = atomicAdd(qn, __popc(m));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (push) {
            const int pos = base + __popc(m & ((1u << lane) - 1u));
            QK[pos] = k;
            QQ[pos] = q;
            QI[pos] = i;
        }
    }
}

// Evaluates work-queue entry e (if valid) in FP32 and appends it to the redo
// queue when its error estimate exceeds tol.
template <int PROC>
__device__ __forceinline__ void fp32_step(Queues<PROC> &s, int e, bool valid, double *out,
                                          const noa_dcs_consts &c, float tol) {
    bool redo = false;
    double k = 0., q = 0.;
    int64_t i = 0;
    if (valid) {
        k = s.wK[e];
        q = s.wQ[e];
        i = s.wI[e];
        float est;
        const double v = eval32<PROC>(k, q, c, est);
        redo = !(est <= tol);
        if (!redo)
            out[i] = v;
    }
    push_queue(redo, k, q, i, s.rK, s.rQ, s.rI, &s.rn);
}

// Pair production: evaluates redo-queue entry e (if valid) with the
// float-float screening log and appends it to the third queue when its
// estimate still exceeds tol.
template <int PROC>
__device__ __forceinline__ void fine_step(Queues<PROC> &s, int e, bool valid, double *out,
                                          const noa_dcs_consts &c, float tol) {
    bool redo = false;
    double k = 0., q = 0.;
    int64_t i = 0;
    if (valid) {
        k = s.rK[e];
        q = s.rQ[e];
        i = s.rI[e];
        float est;
        const double v = pprod_fp32c<false, true>(k, q, c, est);
        redo = !(est <= tol);
        if (!redo)
            out[i] = v;
    }
    push_queue(redo, k, q, i, s.xK, s.xQ, s.xI, &s.xn);
}

template <int PROC>
__global__ void __launch_bounds__(F_THREADS, f32_min_ctas<PROC>()) dcs_fp32c_kernel(const double *__restrict__ K,
                                                              const double *__restrict__ q, double *out, int64_t n,
                                                              const noa_dcs_consts c, float tol) {
    __shared__ Queues<PROC> s;
    if (threadIdx.x == 0) {
        s.rn = 0;
        s.xn = 0;
    }
    int qn = 0;
    int64_t base = (int64_t)blockIdx.x * F_TILE;
    for (;;) {
        const bool more = base < n;  // block-uniform
        if (more) {
            double k[F_ITEMS], r[F_ITEMS];
            unsigned open = 0;
#pragma unroll
            for (int j = 0; j < F_ITEMS; j++) {
                const int64_t i = base + j * F_THREADS + threadIdx.x;
                if (i < n) {
                    k[j] = K[i];
                    r[j] = q[i];
                    if (open32<PROC>(k[j], r[j], c))
                        open |= 1u << j;
                    else
                        out[i] = 0.;
                }
            }
            int pos = qn + scan_block(__popc(open), s.warp_tot, &s.tile_open);
#pragma unroll
            for (int j = 0; j < F_ITEMS; j++) {
                if (open & (1u << j)) {
                    s.wK[pos] = k[j];
                    s.wQ[pos] = r[j];
                    s.wI[pos] = base + j * F_THREADS + threadIdx.x;
                    pos++;
                }
            }
            __syncthreads();
            qn += s.tile_open;
            base += (int64_t)gridDim.x * F_TILE;
        }
        // One call site each for the FP32 step, the redo step and the FP64
        // evaluation (see the FP64 kernels): full batches while tiles remain,
        // everything at the end.
        for (;;) {
            bool did = false;
            if (qn >= F_THREADS || (!more && qn > 0)) {
                const int take = qn < F_THREADS ? qn : F_THREADS;
                fp32_step<PROC>(s, qn - take + threadIdx.x, (int)threadIdx.x < take, out, c, tol);
                qn -= take;
                did = true;
            }
            __syncthreads();
            const int rn = s.rn;
            if (rn >= F_THREADS || (!more && qn == 0 && rn > 0)) {
                const int take = rn < F_THREADS ? rn : F_THREADS;
                if (PROC == NOA_DCS_PROC_PPROD) {
                    fine_step<PROC>(s, rn - take + threadIdx.x, (int)threadIdx.x < take, out, c, tol);
                } else if ((int)threadIdx.x < take) {
                    const int e = rn - take + threadIdx.x;
                    out[s.rI[e]] = redo64<PROC>(s.rK[e], s.rQ[e], c);
                }
                __syncthreads();
                if (threadIdx.x == 0)
                    s.rn = rn - take;
                __syncthreads();
                did = true;
            }
            if (PROC == NOA_DCS_PROC_PPROD) {
                const int xn = s.xn;
                if (xn >= F_THREADS || (!more && qn == 0 && s.rn == 0 && xn > 0)) {
                    const int take = xn < F_THREADS ? xn : F_THREADS;
                    if ((int)threadIdx.x < take) {
                        const int e = xn - take + threadIdx.x;
                        out[s.xI[e]] = redo64<PROC>(s.xK[e], s.xQ[e], c);
                    }
                    __syncthreads();
                    if (threadIdx.x == 0)
                        s.xn = xn - take;
                    __syncthreads();
                    did = true;
                }
            }
            if (!did)
                break;
        }
        if (!more)
            break;
    }
}

static int sm_count() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

template <int PROC>
static cudaError_t launch(const double *K, const double *q, double *out, int64_t n, const noa_dcs_consts &c,
                          float tol, cudaStream_t s) {
    const int64_t tiles = (n + F_TILE - 1) / F_TILE;
    const int64_t cap = (int64_t)sm_count() * 4;
    const int grid = (int)(tiles < cap ? tiles : cap);
    dcs_fp32c_kernel<PROC><<<grid, F_THREADS, 0, s>>>(K, q, out, n, c, tol);
    return cudaGetLastError();
}

} // namespace noa_dcs

using namespace noa_dcs;

cudaError_t noa_dcs_launch_fp32c(int process, const double *K, const double *q, double *out, int64_t n,
                                 const noa_dcs_consts *c, float tol, cudaStream_t stream) {
    if (n <= 0)
        return cudaSuccess;
    switch (process) {
    case NOA_DCS_PROC_BREMS:
        return launch<NOA_DCS_PROC_BREMS>(K, q, out, n, *c, tol, stream);
    case NOA_DCS_PROC_PPROD:
        return launch<NOA_DCS_PROC_PPROD>(K, q, out, n, *c, tol, stream);
    case NOA_DCS_PROC_PHOTO:
        return launch<NOA_DCS_PROC_PHOTO>(K, q, out, n, *c, tol, stream);
    case NOA_DCS_PROC_ION:
        return launch<NOA_DCS_PROC_ION>(K, q, out, n, *c, tol, stream);
    default:
        return cudaErrorInvalidValue;
    }
}
