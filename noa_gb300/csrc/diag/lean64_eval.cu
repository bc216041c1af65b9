/*
 * Diagnostics entry point of libnoa_dcs_diag.so: evaluates one lean64 function (lean64.cuh), one
 * integer-pipe conversion (fpconv.cuh) or one float-float function
 * (dcs_fp32c.cuh) element-wise so that tests can bound its error against a
 * host libm, or check it bit for bit against the cast it replaces.  No
 * counterpart in the reference.
 */
#include "noa_dcs_diag.h"

#include "../dcs_fp32c.cuh"
#include "../dcs_launch.h"
#include "../lean64.cuh"

#include <initializer_list>

namespace {

__global__ void lean64_eval_kernel(int fn, const double *__restrict__ x, const double *__restrict__ y, double *out,
                                   int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double a = x[i];
        double r;
        switch (fn) {
        case 0: r = lean64::lean_log(a); break;
        case 1: r = lean64::lean_exp(a); break;
        case 2: r = lean64::lean_rcp(a); break;
        case 3: r = lean64::lean_div(a, y[i]); break;
        case 4: r = lean64::lean_sqrt(a); break;
        case 5: r = fpconv::f64(fpconv::f32(a)); break;      // (double)(float)a
        case 6: r = fpconv::f64i(__double2int_rz(a)); break;  // (double)(int)a
        case 7: r = noa_dcs::ff_to_double(noa_dcs::ff_exp(noa_dcs::ff_from(a))); break;
        case 8: r = noa_dcs::ff_to_double(noa_dcs::ff_log(noa_dcs::ff_from(a))); break;
        default: r = fpconv::f64(fpconv::f32_normal(a)); break;  // (double)(float)a or NaN
        }
        out[i] = r;
    }
}

} // namespace

extern "C" int noa_dcs_lean64_eval(int fn, const double *x, const double *y, double *out, int64_t n, void *stream) {
    if (fn < 0 || fn > 9 || n < 0 || (n > 0 && (!x || !out || (fn == 3 && !y))))
        return NOA_DCS_ERROR_INVALID_VALUE;
    if (n == 0)
        return NOA_DCS_SUCCESS;
    int dev = 0;
    cudaGetDevice(&dev);
    for (const void *ptr : {(const void *)x, (const void *)out, (const void *)(fn == 3 ? y : x)}) {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
            cudaGetLastError();
            return NOA_DCS_ERROR_NOT_DEVICE_MEMORY;
        }
        if (!(a.type == cudaMemoryTypeManaged || (a.type == cudaMemoryTypeDevice && a.device == dev)))
            return NOA_DCS_ERROR_NOT_DEVICE_MEMORY;
    }
    const int64_t blocks = (n + 255) / 256;
    lean64_eval_kernel<<<(int)(blocks < 4096 ? blocks : 4096), 256, 0, (cudaStream_t)stream>>>(fn, x, y, out, n);
    return cudaGetLastError() == cudaSuccess ? NOA_DCS_SUCCESS : NOA_DCS_ERROR_CUDA;
}
