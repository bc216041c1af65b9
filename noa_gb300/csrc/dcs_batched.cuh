/*
 * Batched multi-element DCS engine: one persistent launch evaluates one
 * process for up to NOA_DCS_MAX_SEGMENTS elements, each with its own
 * (uneven) number of pairs, stored back to back in K, q and result.
 *
 *  - Work unit: a tile of THREADS x items consecutive pairs of one segment.
 *    Tiles of all segments form one index space (prefix sums in the
 *    parameters); each CTA takes the next tile from a global counter
 *    (atomicAdd), so CTAs balance across the uneven segments without a
 *    host-side split.  The counter is the engine's only global scratch and is
 *    zeroed by a memset node before each launch.
 *  - Inside a CTA the tile goes through the same compaction as the
 *    single-element kernels: open pairs are appended to a shared-memory work
 *    queue that is popped 256 (THREADS) at a time; for FP32C, pairs whose error
 *    estimate exceeds the tolerance go to a redo queue evaluated in FP64
 *    (pair production: evaluated again with its screening log in float-float
 *    arithmetic, and only what that still rejects in FP64).
 *    When the next tile belongs to another segment the queues are drained
 *    first, so every warp evaluates pairs of a single element and the element
 *    constants stay warp-uniform (they are read from the parameter space).
 *  - THREADS is a template parameter (128 or 256), items per thread (1-8) and
 *    CTAs per SM are launch parameters: the autotuner's search space.
 *
 * No counterpart in the reference, which evaluates one element per call.
 */
#pragma once

#include "dcs_fp32c.cuh"
#include "dcs_fp64.cuh"
#include "dcs_launch.h"

#include <atomic>

namespace noa_dcs {

struct BatchParams {
    const double *K;
    const double *q;
    double *out;
    unsigned long long *counter;
    int n_seg;
    int items;
    float tol;
    int pad_;
    int64_t seg_begin[NOA_DCS_MAX_SEGMENTS + 1];
    int64_t tile_begin[NOA_DCS_MAX_SEGMENTS + 1];
    noa_dcs_consts consts[NOA_DCS_MAX_SEGMENTS];
};

template <int PROC>
__device__ __forceinline__ bool batch_open(double K, double q, const noa_dcs_consts &c) {
    if (PROC == NOA_DCS_PROC_PPROD)
        return pprod_live(K, q, c);
    else if (PROC == NOA_DCS_PROC_PHOTO)
        return photo_live(K, q, c);
    else
        return true;
}

template <int PROC>
__device__ __forceinline__ double batch_eval64(double K, double q, const noa_dcs_consts &c) {
    if (PROC == NOA_DCS_PROC_BREMS)
        return brems_fp64(K, q, c);
    else if (PROC == NOA_DCS_PROC_PPROD)
        return pprod_fp64(K, q, c);
    else if (PROC == NOA_DCS_PROC_PHOTO)
        return photo_fp64(K, q, c);
    else
        return ion_fp64(K, q, c);
}

// The FP32C engine's FP64 redo: out of line for the two quadrature processes.
template <int PROC>
__device__ __forceinline__ double batch_redo64(double K, double q, const noa_dcs_consts &c) {
    if (PROC == NOA_DCS_PROC_PPROD)
        return pprod_fp64_ol(K, q, c);
    else if (PROC == NOA_DCS_PROC_PHOTO)
        return photo_fp64_ol(K, q, c);
    return batch_eval64<PROC>(K, q, c);
}

template <int PROC>
__device__ __forceinline__ double batch_eval32(double K, double q, const noa_dcs_consts &c, float &est) {
    if (PROC == NOA_DCS_PROC_BREMS)
        return brems_fp32c(K, q, c, est);
    else if (PROC == NOA_DCS_PROC_PPROD)
        return pprod_fp32c<false>(K, q, c, est);
    else if (PROC == NOA_DCS_PROC_PHOTO)
        return photo_fp32c<false>(K, q, c, est);
    else
        return ion_fp32c(K, q, c, est);
}

template <int THREADS>
__device__ __forceinline__ int batch_scan(int v, int *warp_tot, int *total) {
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
        const int w = lane < (THREADS >> 5) ? warp_tot[lane] : 0;
        int s = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o)
                s += y;
        }
        if (lane < (THREADS >> 5))
            warp_tot[lane] = s - w;
        if (lane == 31)
            *total = s;
    }
    __syncthreads();
    return warp_tot[warp] + x - v;
}

// Shared memory of one CTA: work queue of capacity items*THREADS + THREADS,
// then the redo queue (2*THREADS), then for FP32C pair production the third
// queue (2*THREADS) of the pairs its float-float redo step still rejects, as
// dynamic shared memory.
template <int THREADS>
struct BatchSmem {
    static __host__ __device__ size_t bytes(int items, bool third) {
        return (size_t)(items * THREADS + THREADS) * 24 + (size_t)(2 * THREADS) * 24 +
               (third ? (size_t)(2 * THREADS) * 24 : 0);
    }
};

__host__ __device__ constexpr bool batch_third_queue(int proc, int prec) {
    return proc == NOA_DCS_PROC_PPROD && prec != NOA_DCS_FP64;
}

// Appends (k, q, i) of the lanes with `push` to a queue (warp-aggregated).
__device__ __forceinline__ void batch_push(bool push, double k, double q, int64_t i, double *QK, double *QQ,
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

// Pair production, FP32C: evaluates redo-queue entry e (if valid) with the
// float-float screening log; pairs whose estimate still exceeds tol go to the
// third queue.
__device__ __forceinline__ void batch_fine_step(double *rK, double *rQ, int64_t *rI, double *xK, double *xQ,
                                                int64_t *xI, int *xn, int e, bool valid, double *out,
                                                const noa_dcs_consts &c, float tol) {
    bool redo = false;
    double k = 0., q = 0.;
    int64_t i = 0;
    if (valid) {
        k = rK[e];
        q = rQ[e];
        i = rI[e];
        float est;
        const double v = pprod_fp32c<false, true>(k, q, c, est);
        redo = !(est <= tol);
        if (!redo)
            out[i] = v;
    }
    batch_push(redo, k, q, i, xK, xQ, xI, xn);
}

// One evaluation step over work-queue entry e: FP64 writes directly; FP32C
// writes or appends to the redo queue.
template <int PROC, int PREC>
__device__ __forceinline__ void batch_step(double *wK, double *wQ, int64_t *wI, double *rK, double *rQ,
                                           int64_t *rI, int *rn, int e, bool valid, double *out,
                                           const noa_dcs_consts &c, float tol) {
    if (PREC == NOA_DCS_FP64) {
        if (valid)
            out[wI[e]] = batch_eval64<PROC>(wK[e], wQ[e], c);
        return;
    }
    bool redo = false;
    double k = 0., q = 0.;
    int64_t i = 0;
    if (valid) {
        k = wK[e];
        q = wQ[e];
        i = wI[e];
        float est;
        const double v = batch_eval32<PROC>(k, q, c, est);
        redo = !(est <= tol);
        if (!redo)
            out[i] = v;
    }
    batch_push(redo, k, q, i, rK, rQ, rI, rn);
}

template <int PROC, int PREC, int THREADS>
__global__ void __launch_bounds__(THREADS) dcs_batched_kernel(const __grid_constant__ BatchParams p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int items = p.items;
    const int qcap = items * THREADS + THREADS;
    double *wK = reinterpret_cast<double *>(smem_raw);
    double *wQ = wK + qcap;
    int64_t *wI = reinterpret_cast<int64_t *>(wQ + qcap);
    double *rK = reinterpret_cast<double *>(wI + qcap);
    double *rQ = rK + 2 * THREADS;
    int64_t *rI = reinterpret_cast<int64_t *>(rQ + 2 * THREADS);
    double *xK = reinterpret_cast<double *>(rI + 2 * THREADS);  // third queue (batch_third_queue only)
    double *xQ = xK + 2 * THREADS;
    int64_t *xI = reinterpret_cast<int64_t *>(xQ + 2 * THREADS);
    constexpr bool third = batch_third_queue(PROC, PREC);
    __shared__ int warp_tot[THREADS / 32];
    __shared__ int tile_open;
    __shared__ int rn, xn;
    __shared__ unsigned long long s_tile;

    const int tile_size = items * THREADS;
    const long long total_tiles = p.tile_begin[p.n_seg];
    if (threadIdx.x == 0) {
        rn = 0;
        xn = 0;
    }
    int qn = 0;
    int cur = -1;
    for (;;) {
        if (threadIdx.x == 0)
            s_tile = atomicAdd(p.counter, 1ULL);
        __syncthreads();
        const long long tile = (long long)s_tile;
        __syncthreads();
        const bool done = tile >= total_tiles;
        int seg = cur < 0 ? 0 : cur;
        if (!done) {
            while (seg + 1 < p.n_seg && tile >= p.tile_begin[seg + 1])
                seg++;
            while (seg > 0 && tile < p.tile_begin[seg])
                seg--;
        }
        if (cur >= 0) {
            // Drain the queues of the current element: full batches, or
            // everything when the element changes or the work is done.  One
            // call site each for the step and the redo, so that a pair's result
            // does not depend on where it sits in the queue (nvcc may contract
            // differently in separately inlined copies).
            const bool flush = done || seg != cur;
            const noa_dcs_consts &cc = p.consts[cur];
            for (;;) {
                bool did = false;
                if (qn >= THREADS || (flush && qn > 0)) {
                    const int take = qn < THREADS ? qn : THREADS;
                    batch_step<PROC, PREC>(wK, wQ, wI, rK, rQ, rI, &rn, qn - take + threadIdx.x,
                                           (int)threadIdx.x < take, p.out, cc, p.tol);
                    qn -= take;
                    did = true;
                }
                __syncthreads();
                if (PREC != NOA_DCS_FP64) {
                    const int r = rn;
                    if (r >= THREADS || (flush && qn == 0 && r > 0)) {
                        const int take = r < THREADS ? r : THREADS;
                        if (third) {
                            batch_fine_step(rK, rQ, rI, xK, xQ, xI, &xn, r - take + threadIdx.x,
                                            (int)threadIdx.x < take, p.out, cc, p.tol);
                        } else if ((int)threadIdx.x < take) {
                            const int e = r - take + threadIdx.x;
                            p.out[rI[e]] = batch_redo64<PROC>(rK[e], rQ[e], cc);
                        }
                        __syncthreads();
                        if (threadIdx.x == 0)
                            rn = r - take;
                        __syncthreads();
                        did = true;
                    }
                }
                if (third) {
                    const int x = xn;
                    if (x >= THREADS || (flush && qn == 0 && rn == 0 && x > 0)) {
                        const int take = x < THREADS ? x : THREADS;
                        if ((int)threadIdx.x < take) {
                            const int e = x - take + threadIdx.x;
                            p.out[xI[e]] = batch_redo64<PROC>(xK[e], xQ[e], cc);
                        }
                        __syncthreads();
                        if (threadIdx.x == 0)
                            xn = x - take;
                        __syncthreads();
                        did = true;
                    }
                }
                if (!did)
                    break;
            }
        }
        if (done)
            break;
        cur = seg;
        const noa_dcs_consts &c = p.consts[seg];
        const int64_t seg_end = p.seg_begin[seg + 1];
        const int64_t base = p.seg_begin[seg] + (int64_t)(tile - p.tile_begin[seg]) * tile_size;

        double k[8], r[8];
        unsigned open = 0;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            if (j < items) {
                const int64_t i = base + j * THREADS + threadIdx.x;
                if (i < seg_end) {
                    k[j] = p.K[i];
                    r[j] = p.q[i];
                    if (batch_open<PROC>(k[j], r[j], c))
                        open |= 1u << j;
                    else
                        p.out[i] = 0.;
                }
            }
        }
        int pos = qn + batch_scan<THREADS>(__popc(open), warp_tot, &tile_open);
#pragma unroll
        for (int j = 0; j < 8; j++) {
            if (open & (1u << j)) {
                wK[pos] = k[j];
                wQ[pos] = r[j];
                wI[pos] = base + j * THREADS + threadIdx.x;
                pos++;
            }
        }
        __syncthreads();
        qn += tile_open;
    }
}

// Raises a kernel's dynamic shared-memory limit once per device to the most
// it can take (the device's opt-in maximum less the kernel's static shared
// memory; `done` is the kernel's own flag table), so that only the first
// launch on a device above 48 KB sets a function attribute and later
// launches, including launches inside a caller's stream capture, set none.
constexpr int kSmemOptinDevices = 64;
template <typename Kernel>
inline cudaError_t smem_optin_once(Kernel k, size_t smem, std::atomic<bool> (&done)[kSmemOptinDevices]) {
    if (smem <= 48 * 1024)
        return cudaSuccess;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return e;
    if (dev >= 0 && dev < kSmemOptinDevices && done[dev].load(std::memory_order_acquire))
        return cudaSuccess;
    int optin = 0;
    e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess)
        return e;
    cudaFuncAttributes fa;
    e = cudaFuncGetAttributes(&fa, k);
    if (e != cudaSuccess)
        return e;
    const int max_dynamic = optin - (int)fa.sharedSizeBytes;
    if (max_dynamic <= 0 || smem > (size_t)max_dynamic)
        return cudaErrorInvalidValue;
    e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dynamic);
    if (e == cudaSuccess && dev >= 0 && dev < kSmemOptinDevices)
        done[dev].store(true, std::memory_order_release);
    return e;
}

} // namespace noa_dcs
