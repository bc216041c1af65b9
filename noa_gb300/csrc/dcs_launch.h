/*
 * Internal launch interface between the C ABI (dcs_capi.cu) and the kernel
 * translation units.  Not installed; the public surface is include/noa_dcs.h.
 */
#pragma once

#include "../../include/noa_dcs.h"
#include "dcs_consts.h"

#include <cuda_runtime.h>

#define NOA_DCS_PROC_BREMS NOA_DCS_BREMSSTRAHLUNG
#define NOA_DCS_PROC_PPROD NOA_DCS_PAIR_PRODUCTION
#define NOA_DCS_PROC_PHOTO NOA_DCS_PHOTONUCLEAR
#define NOA_DCS_PROC_ION NOA_DCS_IONISATION

#define NOA_DCS_MAX_SEGMENTS 16

/* FP64 kernels (dcs_fp64.cu).  Arguments are already validated. */
cudaError_t noa_dcs_launch_fp64(int process, const double *K, const double *q, double *out, int64_t n,
                                const noa_dcs_consts *c, cudaStream_t stream);

/* FP32-compensated kernels (dcs_fp32c.cu): pairs whose estimated relative
 * error exceeds tol are recomputed in FP64. */
cudaError_t noa_dcs_launch_fp32c(int process, const double *K, const double *q, double *out, int64_t n,
                                 const noa_dcs_consts *c, float tol, cudaStream_t stream);

/* Default FP32C tolerance: relative error bound per pair. */
#define NOA_DCS_FP32C_DEFAULT_TOL 1e-6f

/* Batched engine (dcs_batched.cuh): launch one instantiation.  params points
 * to a noa_dcs::BatchParams; threads is 128 or 256. */
cudaError_t noa_dcs_batched_launch64(int process, int threads, const void *params, int grid, size_t smem,
                                     cudaStream_t stream);
cudaError_t noa_dcs_batched_launch32(int process, int threads, const void *params, int grid, size_t smem,
                                     cudaStream_t stream);
/* Resident CTAs per SM of one instantiation at the given dynamic smem. */
int noa_dcs_batched_occupancy64(int process, int threads, size_t smem);
int noa_dcs_batched_occupancy32(int process, int threads, size_t smem);

/* Recoil integrals (dcs_integral.cu): moment 0 = DEL, 1 = CEL; min_points in
 * 1..1536 (6 ceil(min_points / 6) nodes per K). */
cudaError_t noa_dcs_launch_recoil_integral(int process, int moment, const double *K, double *out, int64_t n,
                                           double xlow, int min_points, const noa_dcs_consts *c,
                                           cudaStream_t stream);

/* Soft-scattering transverse transport per K (dcs_integral.cu). */
cudaError_t noa_dcs_launch_soft_scattering(const double *K, double *out, int64_t n, const noa_dcs_consts *c,
                                           cudaStream_t stream);

/* Per-element constants of the elastic-scattering kernels, computed on the
 * host with the C library: A13 = pow(A, 1/3), Z23 = pow(Z, 2/3). */
struct noa_coulomb_element {
    double A;
    double A13;
    double Z23;
    int32_t Z;
};

/* Elastic scattering (coulomb.cu).  Arguments are already validated. */
cudaError_t noa_dcs_launch_coulomb_data(const double *K, int64_t n, const noa_coulomb_element *e, double mass,
                                        double *fCM, double *screen, double *fspin, double *invlambda,
                                        cudaStream_t stream);
cudaError_t noa_dcs_launch_coulomb_transport(const double *screen, const double *fspin, const double *mu,
                                             int64_t n_mu, int64_t n, double *coefs, cudaStream_t stream);
cudaError_t noa_dcs_launch_hard_scattering(const double *G, const double *fCM, const double *screen,
                                           const double *invlambda, const double *fspin, int64_t nel, int64_t nkin,
                                           double max_mu0, double *mu0, double *lb_h, cudaStream_t stream);
