/*
 * noa_dcs.h -- C ABI of the GB300 muon differential-cross-section (DCS) library.
 *
 * Drop-in for the GPU surface of NOA's PMS DCS, noa::pms::dcs::cuda
 * (grinisrit/noa src/noa/pms/dcs.hh:1004-1019, implemented in
 * src/noa/pms/dcs.cuh:30-50), which the reference provides for bremsstrahlung
 * only.  Every entry point takes plain pointers and sizes, never throws, never
 * aborts, and returns a noa_dcs_status.  A C++/LibTorch layer
 * (include/noa_gb300/dcs_cuda.hh) and the Python package sit on top of it.
 *
 * Memory and streams: unless a function says otherwise, K, q and result are
 * float64 DEVICE buffers of n elements on the current CUDA device, each
 * 8-byte aligned; result may be the same buffer as K or q (each element is
 * read before it is written) but must not partially overlap either.  Work is
 * enqueued on `stream` (a cudaStream_t; NULL = legacy default stream) and the
 * call returns without synchronising, like the reference's launch
 * (src/noa/utils/common.cuh:45-56).  n == 0 is a no-op.
 */
#ifndef NOA_DCS_H
#define NOA_DCS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NOA_DCS_ABI_VERSION 1

/* Mirrors noa::pms::AtomicElement (src/noa/pms/physics.hh:39-43):
 * A in g/mol, I (mean excitation energy) in GeV, Z the charge number.
 * Same member order and size (24 bytes, 4 trailing pad bytes). */
typedef struct noa_dcs_element {
    double A;
    double I;
    int32_t Z;
} noa_dcs_element;

/* The four processes: physics.hh:114-153, dcs.hh:144-258, dcs.hh:362-405,
 * dcs.hh:408-443. */
typedef enum noa_dcs_process {
    NOA_DCS_BREMSSTRAHLUNG = 0,
    NOA_DCS_PAIR_PRODUCTION = 1,
    NOA_DCS_PHOTONUCLEAR = 2,
    NOA_DCS_IONISATION = 3
} noa_dcs_process;

/* Arithmetic of a launch.  FP64 is the drop-in: it matches the reference's
 * FP64 CPU path to a mean relative error below 1e-12.  FP32C runs the
 * quadrature bodies in FP32 with compensated node sums, keeps FP64 at the
 * kinematic edges and bounds, and recomputes in FP64 every pair whose
 * estimated relative error exceeds the tolerance (1e-6 by default), so its
 * relative error against the FP64 result stays below that tolerance. */
typedef enum noa_dcs_precision {
    NOA_DCS_FP64 = 0,
    NOA_DCS_FP32C = 1
} noa_dcs_precision;

typedef enum noa_dcs_status {
    NOA_DCS_SUCCESS = 0,
    NOA_DCS_ERROR_INVALID_VALUE = 1,     /* bad process / precision / n < 0 / null pointer */
    NOA_DCS_ERROR_INVALID_ELEMENT = 2,   /* A or I not finite and positive, or Z < 1 */
    NOA_DCS_ERROR_MISALIGNED = 3,        /* a buffer is not 8-byte aligned */
    NOA_DCS_ERROR_NOT_DEVICE_MEMORY = 4, /* a buffer is not device memory of the current device */
    NOA_DCS_ERROR_OVERLAP = 5,           /* result partially overlaps K or q */
    NOA_DCS_ERROR_CUDA = 6,              /* a CUDA runtime call failed; see noa_dcs_last_error() */
    NOA_DCS_ERROR_TIMEOUT = 7,           /* a bounded device-side wait expired */
    NOA_DCS_ERROR_NOT_SUPPORTED = 8      /* combination not built (e.g. FP32C for ionisation) */
} noa_dcs_status;

/* ---- per-process entry points: the functions a binding of
 * noa::pms::dcs::cuda::vmap_<process> (dcs.hh:1004-1010, dcs.cuh:30-41)
 * calls.  result[i] = dcs(K[i], q[i], element, mass) in FP64. */
int noa_dcs_cuda_vmap_bremsstrahlung(double *result, const double *K, const double *q, int64_t n,
                                     const noa_dcs_element *element, double mass, void *stream);
int noa_dcs_cuda_vmap_pair_production(double *result, const double *K, const double *q, int64_t n,
                                      const noa_dcs_element *element, double mass, void *stream);
int noa_dcs_cuda_vmap_photonuclear(double *result, const double *K, const double *q, int64_t n,
                                   const noa_dcs_element *element, double mass, void *stream);
int noa_dcs_cuda_vmap_ionisation(double *result, const double *K, const double *q, int64_t n,
                                 const noa_dcs_element *element, double mass, void *stream);

/* Generic form of the four above with a precision selector.  Replaces the
 * dispatch a caller would otherwise write over dcs::vmap(dcs::<process>)
 * (dcs.hh:35-48). */
int noa_dcs_cuda_vmap(int process, int precision, double *result, const double *K, const double *q, int64_t n,
                      const noa_dcs_element *element, double mass, void *stream);

/* Recoil-energy integrals per kinetic energy, the GPU form of
 * dcs::vmap_integral(dcs::recoil_integral(dcs::<process>, integrand))
 * (dcs.hh:89-130, 955-1001):
 *   result[i] = int_{K xlow}^{K} q^(1+moment) dsigma/dq(K, q) dq / (K + mass),
 * K = K[i], moment 0 = DEL (del_integrand), 1 = CEL (cel_integrand), with
 * the reference's composite 6-node Gauss-Legendre rule over log q on
 * ceil(min_points/6) intervals (min_points in 1..1536; the reference's tests
 * use 180, xlow = X_FRACTION = 0.05), and ionisation's closed form below its
 * radiative-correction threshold.  FP64; K and result are device buffers. */
int noa_dcs_cuda_recoil_integral(int process, int moment, double *result, const double *K, int64_t n, double xlow,
                                 const noa_dcs_element *element, double mass, int32_t min_points, void *stream);

/* Soft-scattering transverse transport per kinetic energy, the GPU form of
 * dcs::soft_scattering (dcs.hh:941-952):
 *   result[i] = transverse_transport_ionisation(K[i])      (dcs.hh:874-899)
 *             + transverse_transport_photonuclear(K[i])    (dcs.hh:901-939),
 * the latter a 102-node composite Gauss-Legendre rule over log(nu / 0.05) on
 * [log 1e-6, 0] of the photonuclear DCS times its analytic angular weight.
 * FP64; K and result are device buffers. */
int noa_dcs_cuda_soft_scattering(double *result, const double *K, int64_t n, const noa_dcs_element *element,
                                 double mass, void *stream);

/* Elastic (Coulomb) scattering data per kinetic energy, the GPU form of
 * dcs::coulomb_data (dcs.hh:604-622).  Outputs, in the reference's record
 * layout: fCM [n][2] (CM Lorentz factors), screen [n][9] (three screening
 * parameters and six pole-reduction factors), fspin [n], invlambda [n]
 * (inverse Wentzel path).  FP64, device buffers. */
int noa_dcs_cuda_coulomb_data(double *fCM, double *screen, double *fspin, double *invlambda, const double *K,
                              int64_t n, const noa_dcs_element *element, double mass, void *stream);

/* First two elastic transport coefficients below the cut-off angle mu, the
 * GPU form of dcs::coulomb_transport (dcs.hh:679-699): coefficients [n][2]
 * from screen [n][9] and fspin [n]; mu holds n_mu = 1 (one angle for all)
 * or n values.  FP64, device buffers. */
int noa_dcs_cuda_coulomb_transport(double *coefficients, const double *screen, const double *fspin,
                                   const double *mu, int64_t n_mu, int64_t n, void *stream);

/* Hard-scattering cut-off angle mu0 [nkin] and mean free path lb_h [nkin]
 * over nel elements, the GPU form of dcs::hard_scattering (dcs.hh:840-872,
 * Ridders' root of the restricted cross-section, numerics.hh:154-216).
 * Inputs per element and energy: G [nel][nkin][2] (transport
 * coefficients), fCM [nel][nkin][2], screen [nel][nkin][9], invlambda and
 * fspin [nel][nkin].  FP64, device buffers. */
int noa_dcs_cuda_hard_scattering(double *mu0, double *lb_h, const double *G, const double *fCM,
                                 const double *screen, const double *invlambda, const double *fspin, int64_t nel,
                                 int64_t nkin, void *stream);

/* FP32-compensated form with an explicit tolerance: every pair whose
 * estimated relative error exceeds `tolerance` (0 < tolerance < 1) is
 * recomputed in FP64 (pair production: first in FP32 with its screening log
 * in float-float arithmetic, and in FP64 if that estimate still exceeds
 * `tolerance`).  noa_dcs_cuda_vmap with NOA_DCS_FP32C uses 1e-6.
 * No counterpart in the reference (which has only FP64). */
int noa_dcs_cuda_vmap_fp32c(int process, double *result, const double *K, const double *q, int64_t n,
                            const noa_dcs_element *element, double mass, float tolerance, void *stream);

/* Host-buffer form: K, q and result are HOST buffers.  When all three are
 * page-locked (cudaHostAlloc / cudaHostRegister, e.g. torch pin_memory), the
 * kernels read and write them in place over the CPU-GPU link, with no
 * staging.  Otherwise the call stages the data through device buffers owned
 * by the library, pipelining host-to-device copies, kernels and
 * device-to-host copies in chunks on its own streams.  Either way it returns
 * when result is complete.  This is the GPU counterpart of calling dcs::vmap /
 * dcs::pvmap on CPU tensors (dcs.hh:35-75). */
int noa_dcs_vmap_host(int process, int precision, double *result, const double *K, const double *q, int64_t n,
                      const noa_dcs_element *element, double mass);

/* ---- batched multi-element engine (no counterpart in the reference, which
 * evaluates one element per call).  One persistent launch evaluates one
 * process for n_segments (1..16) elements; segment s has counts[s] pairs
 * stored back to back in K, q and result (device buffers), element
 * elements[s].  CTAs take tiles from a global counter, so uneven segments
 * balance on the GPU.  The plan owns that counter (allocated at creation;
 * execution allocates nothing) and, after the first execute_graph with a
 * given buffer triple, a CUDA graph of the counter reset and the launch.
 * A plan is not thread-safe; executions of one plan on different streams
 * must not overlap. */
typedef struct noa_dcs_batch_plan noa_dcs_batch_plan;

int noa_dcs_batch_plan_create(noa_dcs_batch_plan **plan, int process, int precision, int n_segments,
                              const noa_dcs_element *elements, const int64_t *counts, double mass);
/* Tile shape: threads per CTA (128 or 256), pairs per thread per tile (1..8),
 * resident CTAs per SM (clamped to the occupancy limit). */
int noa_dcs_batch_plan_set_tile(noa_dcs_batch_plan *plan, int threads, int items, int ctas_per_sm);
int noa_dcs_batch_plan_get_tile(const noa_dcs_batch_plan *plan, int *threads, int *items, int *ctas_per_sm);
/* FP32C plans: per-pair relative error tolerance (default 1e-6). */
int noa_dcs_batch_plan_set_tolerance(noa_dcs_batch_plan *plan, float tolerance);
/* Times every tile shape of the search space on the first sample_per_segment
 * pairs of each segment (all pairs if <= 0), on these buffers, and keeps the
 * fastest.  Writes (part of) result. */
int noa_dcs_batch_plan_autotune(noa_dcs_batch_plan *plan, double *result, const double *K, const double *q,
                                void *stream, int64_t sample_per_segment);
/* Enqueues the counter reset and the launch on stream. */
int noa_dcs_batch_plan_execute(noa_dcs_batch_plan *plan, double *result, const double *K, const double *q,
                               void *stream);
/* Same work as one CUDA graph launch (captured on first use per buffer triple). */
int noa_dcs_batch_plan_execute_graph(noa_dcs_batch_plan *plan, double *result, const double *K, const double *q,
                                     void *stream);
int noa_dcs_batch_plan_destroy(noa_dcs_batch_plan *plan);
/* Message of the last failed batch-plan call on this host thread. */
const char *noa_dcs_batch_last_error(void);

/* Allocation-free batched evaluation (no counterpart in the reference): the
 * work of one batch plan execution -- process, precision (FP32C at tolerance
 * 1e-6), segments (at most 16: larger counts of segments are rejected with
 * NOA_DCS_ERROR_INVALID_VALUE) -- without a plan and without allocating
 * anything.  For callers that cannot let a library allocate device memory:
 * an application that hands all of the GPU's memory to its own arena or pool
 * at start-up, so a cudaMalloc from this library would fail or escape its
 * accounting, or a transport code whose stepping loop may not pay for an
 * allocation's device synchronisation.  The engine's one piece of scratch, a
 * tile counter, lives in a 256-byte static device array that every device
 * loading the library keeps until exit; each call zeroes it on `stream`
 * before the launch.  All calls share that array: calls whose work overlaps
 * on the GPU (different streams, or different host threads) race and must be
 * serialised by the caller.  Set-up on the first call on each device: the
 * array's device address is looked up with that device current, and for
 * FP32C pair production (54 KB of shared memory) the kernel's shared-memory
 * limit is raised; later calls make no runtime set-up call.  Tile
 * shape is fixed (256 threads x 4 pairs, 2 CTAs per SM).  Buffers as for the
 * plan. */
int noa_dcs_cuda_vmap_batched_noalloc(int process, int precision, int n_segments, const noa_dcs_element *elements,
                                      const int64_t *counts, double mass, double *result, const double *K,
                                      const double *q, void *stream);

/* ---- learned surrogate (no counterpart in the reference).  A
 * 4 -> 128 -> 128 -> 128 -> 1 SiLU network predicts the residual of log DCS over
 * an analytic baseline for pair production or photonuclear, from the features
 * (log K, log nu, Z/100, log A).  Training runs on the GPU with the library's
 * own BF16 tensor-core forward / backward kernels and Adam.  The parameter
 * vector has NOA_DCS_MLP_NPARAM floats; norm holds 10 floats: feature shifts
 * (4), feature scales (4), residual shift and scale. */
#define NOA_DCS_MLP_NPARAM 33793
typedef struct noa_dcs_mlp noa_dcs_mlp;

int noa_dcs_mlp_create(noa_dcs_mlp **model, int process, int batch);
int noa_dcs_mlp_set_params(noa_dcs_mlp *model, const float *params, const float *adam_m, const float *adam_v,
                           int64_t step, const float *norm);
int noa_dcs_mlp_get_params(noa_dcs_mlp *model, float *params, float *adam_m, float *adam_v, int64_t *step);
/* Training data from the FP64 kernels: for pairs (K[i], q[i]) of element
 * elements[elem[i]], raw features Xraw[i][4], residual R[i] = log DCS - baseline
 * and state[i]: 1 open with DCS > 0, 0 closed by the kinematic bounds, 2 open
 * by the bounds but DCS = 0.  Device buffers; synchronous. */
int noa_dcs_mlp_prepare(int process, const double *K, const double *q, const uint8_t *elem, int64_t n,
                        const noa_dcs_element *elements, int n_elements, double mass, float *Xraw, float *R,
                        uint8_t *valid, void *stream);
/* n_steps Adam steps on batches perm[b*batch .. (b+1)*batch) of the normalised
 * data X[n][4], T[n]; cosine learning-rate decay from lr to lr_final;
 * losses[n_steps] (device, optional) receives each batch's loss. */
int noa_dcs_mlp_train(noa_dcs_mlp *model, const float *X, const float *T, int64_t n, const int32_t *perm,
                      int64_t n_steps, float lr, float lr_final, float *losses, void *stream);
/* Normalised network output for X[n][4] (device buffers). */
int noa_dcs_mlp_predict(noa_dcs_mlp *model, const float *X, float *out, int64_t n, void *stream);
/* Loss and gradient (NOA_DCS_MLP_NPARAM floats, device) of one batch of n rows. */
int noa_dcs_mlp_gradient(noa_dcs_mlp *model, const float *X, const float *T, int n, float *grad, float *loss,
                         void *stream);
int noa_dcs_mlp_destroy(noa_dcs_mlp *model);
const char *noa_dcs_mlp_last_error(void);
/* Surrogate evaluation of n = sum(counts) pairs laid out as for a batch plan
 * (segment s: element elements[s], counts[s] pairs; at most 16 segments,
 * fewer than 2^31 pairs).  trust is the device trust grid
 * uint8[n_segments][64][64] over (log K in [log 1e-3, log 1e6], log nu in
 * [log 1e-7, 0]): pairs in a trusted cell are answered by the network
 * (tcgen05 tensor cores), all others by the FP32C kernel (FP64 above
 * `tolerance`).  Closed pairs get 0.  stats (pinned or host memory, optional)
 * receives {network pairs, fallback pairs, status} when the stream reaches
 * it; status NOA_DCS_ERROR_TIMEOUT reports an expired tensor-core wait.
 * Allocates its pair lists on first use and when n grows.  The lists are one
 * per process: calls whose work overlaps on the GPU (other streams, other
 * host threads) must be ordered by the caller.  K, q, result and trust must be
 * device memory of the current device (NOA_DCS_ERROR_NOT_DEVICE_MEMORY). */
int noa_dcs_mlp_infer(noa_dcs_mlp *model, const uint8_t *trust, int n_segments, const noa_dcs_element *elements,
                      const int64_t *counts, double mass, double *result, const double *K, const double *q,
                      float tolerance, unsigned long long *stats, void *stream);
const char *noa_dcs_mlp_infer_last_error(void);
/* Accessor used by the inference kernels of this library. */
int noa_dcs_mlp_handles(noa_dcs_mlp *model, int *process, const float **params, const void **weights_bf16,
                        const float **norm);

/* Frees the host-path staging buffers of the current device (they are
 * otherwise kept for reuse until the process exits). */
int noa_dcs_release_staging(void);

/* Human-readable name of a status code (static storage). */
const char *noa_dcs_status_string(int status);

/* Message of the last failed call on this host thread ("" if none). */
const char *noa_dcs_last_error(void);

/* NOA_DCS_ABI_VERSION of the loaded library. */
int noa_dcs_abi_version(void);

#ifdef __cplusplus
}
#endif

#endif /* NOA_DCS_H */
