/*
 * Decision check of libnoa_dcs_diag.so: for each (K, q) pair, a decision
 * that a DCS kernel takes in float or lean arithmetic first -- which pairs
 * are open (pair production, photonuclear), whether bremsstrahlung's
 * electron term exists, whether ionisation's first exit is taken -- beside
 * the reference's exact IEEE decision on the same device, so that tests can
 * place pairs at every bound and require that the two never disagree.  No
 * counterpart in the reference.
 */
#include "noa_dcs_diag.h"

#include "../dcs_fp64.cuh"
#include "../dcs_launch.h"

#include <initializer_list>

namespace {

using namespace noa_dcs;

// out: 1 / 0 the decision (open, electron term, first exit not taken), -1
// ionisation undecided in float (the exact test decides), -2 the fast
// decision disagrees with the exact one.
__global__ void decision_kernel(int proc, const double *__restrict__ K, const double *__restrict__ q, double *out,
                                int64_t n, const noa_dcs_consts c) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double k = K[i], x = q[i];
        double r;
        if (proc == NOA_DCS_PROC_BREMS) {
            const double E = k + c.mass;
            const bool fast = brems_below(E, x, c), exact = brems_below_qe(E, x, c);
            r = fast == exact ? (double)fast : -2.;
        } else if (proc == NOA_DCS_PROC_PPROD) {
            bool exact = !(x <= 4. * ME) && !(x >= k + c.pp_kmax_shift);
            if (exact) {
                const double a = pprod_argmin_exact(k, x, c);
                exact = !((a >= 1.) || (a <= 0.));
            }
            const bool fast = pprod_live(k, x, c);
            r = fast == exact ? (double)fast : -2.;
        } else if (proc == NOA_DCS_PROC_PHOTO) {
            double a, b;
            const bool exact = photo_window(k, x, c, a, b), fast = photo_live(k, x, c);
            r = fast == exact ? (double)fast : -2.;
        } else {
            const double E = k + c.mass, P2 = k * (k + 2. * c.mass);
            const double W = ion_wmax(P2, E, c);
            const int taken = ((W < NOA_X_FRACTION * k) || (x > W)) ? 0 : 1;
            const int first = ion_first_exit(k, x, c);
            r = first < 0 ? -1. : (first == taken ? (double)first : -2.);
        }
        out[i] = r;
    }
}

} // namespace

extern "C" int noa_dcs_decision_check(int proc, const double *K, const double *q, double *out, int64_t n, double A,
                                      double I, int32_t Z, double mass, void *stream) {
    if (proc < 0 || proc > 3 || n < 0 || (n > 0 && (!K || !q || !out)))
        return NOA_DCS_ERROR_INVALID_VALUE;
    if (!(A > 0.) || !(I > 0.) || Z < 1 || !(mass > 0.))
        return NOA_DCS_ERROR_INVALID_VALUE;
    if (n == 0)
        return NOA_DCS_SUCCESS;
    int dev = 0;
    cudaGetDevice(&dev);
    for (const void *ptr : {(const void *)K, (const void *)q, (const void *)out}) {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
            cudaGetLastError();
            return NOA_DCS_ERROR_NOT_DEVICE_MEMORY;
        }
        if (!(a.type == cudaMemoryTypeManaged || (a.type == cudaMemoryTypeDevice && a.device == dev)))
            return NOA_DCS_ERROR_NOT_DEVICE_MEMORY;
    }
    noa_dcs_consts c;
    noa_dcs_fill_consts(&c, A, I, Z, mass);
    const int64_t blocks = (n + 255) / 256;
    decision_kernel<<<(int)(blocks < 4096 ? blocks : 4096), 256, 0, (cudaStream_t)stream>>>(proc, K, q, out, n, c);
    return cudaGetLastError() == cudaSuccess ? NOA_DCS_SUCCESS : NOA_DCS_ERROR_CUDA;
}
