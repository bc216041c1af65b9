/*
 * FP64 muon DCS kernels for sm_103a.
 *
 * Two launch shapes:
 *
 *  - map kernel (bremsstrahlung, ionisation): every pair is live or nearly so
 *    and the body is short, so each thread evaluates ITEMS pairs of a
 *    block-contiguous tile with coalesced loads and stores.
 *
 *  - compacting kernel (pair production, photonuclear): ~46% / ~80% of the
 *    pairs of the seeded workload are closed kinematically and the live ones
 *    run an 8- or 9-node quadrature.  A CTA classifies a tile with the cheap
 *    bound checks (the reference's early returns), writes the zeros straight
 *    away, and appends the live pairs (K, q, index) to a queue in shared
 *    memory.  Whenever the queue holds a full CTA's worth of work, every
 *    thread pops one pair and runs the quadrature, so all 32 lanes of a warp
 *    take the same trip through the node loop.  The remainder is drained after
 *    the last tile.  This is the warp-uniform regime grouping of the hot path;
 *    it needs no global scratch.
 *
 * Each kernel calls the evaluation from exactly one place.  nvcc inlines
 * every call site separately and may contract a * b + c into an FMA
 * differently in each copy, so two call sites (a full-batch drain and a tail,
 * or an unrolled item loop) could round the same pair differently depending
 * on where it sits in the queue.  With one call site a pair's result depends
 * on (K, q) only.
 *
 * The reference launches one thread per pair on the legacy stream
 * (common.cuh:33-56) and recomputes three pow() per bremsstrahlung evaluation
 * (physics.hh:126-128); it has no GPU pair-production, photonuclear or
 * ionisation kernel.
 */
#include "dcs_fp64.cuh"
#include "dcs_launch.h"

#include <cuda_runtime.h>

namespace noa_dcs {

constexpr int MAP_THREADS = 256;
constexpr int MAP_ITEMS = 4;
constexpr int CMP_THREADS = 256;
constexpr int CMP_ITEMS = 4;
constexpr int CMP_TILE = CMP_THREADS * CMP_ITEMS;
constexpr int CMP_QCAP = CMP_TILE + CMP_THREADS;

// Resident CTAs per SM that the compacting kernels are compiled for (the
// register budget per thread follows).  Measured on 1e8 pairs: pair
// production 82.1 ms at 2 (108 registers) against 89.4 ms at 3 and 82.1 ms
// at 1; photonuclear 45.0 ms at 4 (64 registers) against 47.6 ms at 3,
// 45.2 ms at 5 and 46.0 ms at 2.
#define NOA_DCS_PPROD_MIN_CTAS 2
#define NOA_DCS_PHOTO_MIN_CTAS 4

template <int PROC>
__device__ __forceinline__ double eval_fp64(double K, double q, const noa_dcs_consts &c) {
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
__device__ __forceinline__ bool live_fp64(double K, double q, const noa_dcs_consts &c) {
    if (PROC == NOA_DCS_PROC_PPROD)
        return pprod_live(K, q, c);
    else
        return photo_live(K, q, c);
}

template <int PROC>
__global__ void __launch_bounds__(MAP_THREADS) dcs_fp64_map_kernel(const double *__restrict__ K,
                                                                   const double *__restrict__ q, double *out,
                                                                   int64_t n, const noa_dcs_consts c) {
    const int64_t tile = (int64_t)MAP_THREADS * MAP_ITEMS;
    for (int64_t base = (int64_t)blockIdx.x * tile; base < n; base += (int64_t)gridDim.x * tile) {
#pragma unroll 1  // one inlined copy of the evaluation
        for (int j = 0; j < MAP_ITEMS; j++) {
            const int64_t i = base + j * MAP_THREADS + threadIdx.x;
            const double v = eval_fp64<PROC>(i < n ? K[i] : 1., i < n ? q[i] : 1., c);
            if (i < n)
                out[i] = v;
        }
    }
}

// Block-wide exclusive scan of one small count per thread.
__device__ __forceinline__ int block_exclusive_scan(int v, int *warp_tot, int *total) {
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
        int w = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
        int s = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o)
                s += y;
        }
        if (lane < (int)(blockDim.x >> 5))
            warp_tot[lane] = s - w;
        if (lane == 31)
            *total = s;
    }
    __syncthreads();
    return warp_tot[warp] + x - v;
}

template <int PROC>
__global__ void __launch_bounds__(CMP_THREADS, PROC == NOA_DCS_PROC_PHOTO ? NOA_DCS_PHOTO_MIN_CTAS : NOA_DCS_PPROD_MIN_CTAS) dcs_fp64_compact_kernel(const double *__restrict__ K,
                                                                       const double *__restrict__ q, double *out,
                                                                       int64_t n, const noa_dcs_consts c) {
    __shared__ double qK[CMP_QCAP];
    __shared__ double qQ[CMP_QCAP];
    __shared__ int64_t qI[CMP_QCAP];
    __shared__ int warp_tot[CMP_THREADS / 32];
    __shared__ int tile_live;
    int qn = 0; // queue length, identical in every thread
    int64_t base = (int64_t)blockIdx.x * CMP_TILE;
    for (;;) {
        const bool more = base < n;  // block-uniform
        if (more) {
            double k[CMP_ITEMS], r[CMP_ITEMS];
            unsigned live = 0;
#pragma unroll
            for (int j = 0; j < CMP_ITEMS; j++) {
                const int64_t i = base + j * CMP_THREADS + threadIdx.x;
                if (i < n) {
                    k[j] = K[i];
                    r[j] = q[i];
                    if (live_fp64<PROC>(k[j], r[j], c))
                        live |= 1u << j;
                    else
                        out[i] = 0.;
                }
            }
            const int mine = __popc(live);
            int pos = qn + block_exclusive_scan(mine, warp_tot, &tile_live);
#pragma unroll
            for (int j = 0; j < CMP_ITEMS; j++) {
                if (live & (1u << j)) {
                    qK[pos] = k[j];
                    qQ[pos] = r[j];
                    qI[pos] = base + j * CMP_THREADS + threadIdx.x;
                    pos++;
                }
            }
            __syncthreads();
            qn += tile_live;
            base += (int64_t)gridDim.x * CMP_TILE;
        }
        // full batches while tiles remain, then the remainder: one call site
        while (qn >= CMP_THREADS || (!more && qn > 0)) {
            const int take = qn < CMP_THREADS ? qn : CMP_THREADS;
            if ((int)threadIdx.x < take) {
                const int e = qn - take + threadIdx.x;
                out[qI[e]] = eval_fp64<PROC>(qK[e], qQ[e], c);
            }
            qn -= take;
            __syncthreads();
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
static cudaError_t launch_map(const double *K, const double *q, double *out, int64_t n, const noa_dcs_consts &c,
                              cudaStream_t s) {
    const int64_t tile = (int64_t)MAP_THREADS * MAP_ITEMS;
    const int64_t tiles = (n + tile - 1) / tile;
    const int64_t cap = (int64_t)sm_count() * 8;
    const int grid = (int)(tiles < cap ? tiles : cap);
    dcs_fp64_map_kernel<PROC><<<grid, MAP_THREADS, 0, s>>>(K, q, out, n, c);
    return cudaGetLastError();
}

template <int PROC>
static cudaError_t launch_compact(const double *K, const double *q, double *out, int64_t n,
                                  const noa_dcs_consts &c, cudaStream_t s) {
    const int64_t tiles = (n + CMP_TILE - 1) / CMP_TILE;
    const int64_t cap = (int64_t)sm_count() * 4;
    const int grid = (int)(tiles < cap ? tiles : cap);
    dcs_fp64_compact_kernel<PROC><<<grid, CMP_THREADS, 0, s>>>(K, q, out, n, c);
    return cudaGetLastError();
}

} // namespace noa_dcs

using namespace noa_dcs;

cudaError_t noa_dcs_launch_fp64(int process, const double *K, const double *q, double *out, int64_t n,
                                const noa_dcs_consts *c, cudaStream_t stream) {
    if (n <= 0)
        return cudaSuccess;
    switch (process) {
    case NOA_DCS_PROC_BREMS:
        return launch_map<NOA_DCS_PROC_BREMS>(K, q, out, n, *c, stream);
    case NOA_DCS_PROC_PPROD:
        return launch_compact<NOA_DCS_PROC_PPROD>(K, q, out, n, *c, stream);
    case NOA_DCS_PROC_PHOTO:
        return launch_compact<NOA_DCS_PROC_PHOTO>(K, q, out, n, *c, stream);
    case NOA_DCS_PROC_ION:
        return launch_map<NOA_DCS_PROC_ION>(K, q, out, n, *c, stream);
    default:
        return cudaErrorInvalidValue;
    }
}
