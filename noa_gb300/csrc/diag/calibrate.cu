/*
 * Arithmetic-throughput probes that give the roofline denominators of the DCS
 * kernels, which are bound by the FP64 (plain form) and FP32 (compensated
 * form) pipes rather than by HBM or the tensor cores.  Each thread runs
 * CHAINS independent fused multiply-add chains; the result is stored so the
 * chains cannot be removed.  flops = 2 * CHAINS * iters * threads.
 * These kernels have no counterpart in the reference.
 */
#include "noa_dcs_diag.h"

#include "../../../include/noa_dcs.h"

#include <cuda_runtime.h>

namespace {

constexpr int CHAINS = 8;

template <typename T>
__global__ void __launch_bounds__(256) fma_chains(T *out, int iters, T b, T c) {
    T a[CHAINS];
#pragma unroll
    for (int k = 0; k < CHAINS; k++)
        a[k] = (T)(threadIdx.x + k) * (T)1e-3;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < CHAINS; k++)
            a[k] = a[k] * b + c;
    }
    T s = 0;
#pragma unroll
    for (int k = 0; k < CHAINS; k++)
        s += a[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

} // namespace

extern "C" {

/* Launches blocks x 256 threads of FMA chains in FP64 (fp64 != 0) or FP32 on
 * `stream`; out needs blocks*256 elements of that type.  Returns the flop
 * count of the launch through *flops. */
int noa_dcs_probe_fma(int fp64, void *out, int blocks, int iters, double *flops, void *stream) {
    if (!out || blocks <= 0 || iters <= 0)
        return NOA_DCS_ERROR_INVALID_VALUE;
    // out receives blocks x 256 values: it must be device memory of the current device
    int dev = 0;
    cudaPointerAttributes a;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaPointerGetAttributes(&a, out) != cudaSuccess) {
        cudaGetLastError();
        return NOA_DCS_ERROR_NOT_DEVICE_MEMORY;
    }
    if (!(a.type == cudaMemoryTypeManaged || (a.type == cudaMemoryTypeDevice && a.device == dev)))
        return NOA_DCS_ERROR_NOT_DEVICE_MEMORY;
    if (fp64)
        fma_chains<double><<<blocks, 256, 0, (cudaStream_t)stream>>>((double *)out, iters, 0.999999, 1e-7);
    else
        fma_chains<float><<<blocks, 256, 0, (cudaStream_t)stream>>>((float *)out, iters, 0.999999f, 1e-7f);
    if (flops)
        *flops = 2.0 * CHAINS * (double)iters * (double)blocks * 256.0;
    return cudaGetLastError() == cudaSuccess ? NOA_DCS_SUCCESS : NOA_DCS_ERROR_CUDA;
}
}
