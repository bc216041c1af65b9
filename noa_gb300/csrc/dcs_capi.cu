/*
 * C ABI of the GB300 muon DCS library (include/noa_dcs.h): argument checks,
 * per-launch constants, dispatch to the kernels, and the pipelined
 * host-buffer path.
 *
 * The reference checks nothing beyond the dtype check of data_ptr<double>()
 * (src/noa/pms/dcs.cuh:36, common.cuh:47, 65) and ignores launch errors.
 * Here every entry point validates its arguments before any launch (a bad
 * pointer must never reach a kernel), reports CUDA errors as a status, and
 * never throws or aborts.
 */
#include "dcs_launch.h"

#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <initializer_list>
#include <mutex>
#include <utility>

namespace {

thread_local char g_last_error[512] = "";

int fail(int status, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof g_last_error, fmt, ap);
    va_end(ap);
    return status;
}

int cuda_fail(cudaError_t e, const char *what) {
    return fail(NOA_DCS_ERROR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

int check_element(const noa_dcs_element *el) {
    if (!el)
        return fail(NOA_DCS_ERROR_INVALID_VALUE, "element is NULL");
    if (!std::isfinite(el->A) || !(el->A > 0.) || !std::isfinite(el->I) || !(el->I > 0.) || el->Z < 1)
        return fail(NOA_DCS_ERROR_INVALID_ELEMENT, "invalid element A=%g I=%g Z=%d", el->A, el->I, (int)el->Z);
    return NOA_DCS_SUCCESS;
}

int check_common(int process, int precision, int64_t n, double mass) {
    if (process < NOA_DCS_BREMSSTRAHLUNG || process > NOA_DCS_IONISATION)
        return fail(NOA_DCS_ERROR_INVALID_VALUE, "unknown process %d", process);
    if (precision != NOA_DCS_FP64 && precision != NOA_DCS_FP32C)
        return fail(NOA_DCS_ERROR_INVALID_VALUE, "unknown precision %d", precision);
    if (n < 0)
        return fail(NOA_DCS_ERROR_INVALID_VALUE, "negative size %lld", (long long)n);
    if (!std::isfinite(mass) || !(mass > 0.))
        return fail(NOA_DCS_ERROR_INVALID_VALUE, "invalid particle mass %g", mass);
    return NOA_DCS_SUCCESS;
}

bool overlaps_partially(const double *a, const double *b, int64_t n) {
    if (a == b)
        return false;
    const uintptr_t a0 = (uintptr_t)a, a1 = a0 + (uintptr_t)n * 8u;
    const uintptr_t b0 = (uintptr_t)b, b1 = b0 + (uintptr_t)n * 8u;
    return a0 < b1 && b0 < a1;
}

int check_device_buffer(const void *p, const char *name, int device) {
    if (!p)
        return fail(NOA_DCS_ERROR_INVALID_VALUE, "%s is NULL", name);
    if ((uintptr_t)p % 8u)
        return fail(NOA_DCS_ERROR_MISALIGNED, "%s is not 8-byte aligned", name);
    cudaPointerAttributes attr;
    const cudaError_t e = cudaPointerGetAttributes(&attr, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return cuda_fail(e, "cudaPointerGetAttributes");
    }
    if (attr.type != cudaMemoryTypeDevice && attr.type != cudaMemoryTypeManaged)
        return fail(NOA_DCS_ERROR_NOT_DEVICE_MEMORY, "%s is not device memory", name);
    if (attr.type == cudaMemoryTypeDevice && attr.device != device)
        return fail(NOA_DCS_ERROR_NOT_DEVICE_MEMORY, "%s lives on device %d, current device is %d", name,
                    attr.device, device);
    return NOA_DCS_SUCCESS;
}

int launch(int process, int precision, double *result, const double *K, const double *q, int64_t n,
           const noa_dcs_consts *c, cudaStream_t stream, float tol = NOA_DCS_FP32C_DEFAULT_TOL) {
    cudaError_t e;
    if (precision == NOA_DCS_FP64)
        e = noa_dcs_launch_fp64(process, K, q, result, n, c, stream);
    else
        e = noa_dcs_launch_fp32c(process, K, q, result, n, c, tol, stream);
    if (e != cudaSuccess)
        return cuda_fail(e, "kernel launch");
    return NOA_DCS_SUCCESS;
}

// ---------------------------------------------------------------- host path
constexpr int64_t kChunk = (int64_t)1 << 21; // pairs per pipeline stage
constexpr int kSlots = 3;  // copy in, compute and copy out of three chunks overlap
constexpr int kMaxDevices = 64;

struct Staging {
    std::mutex mu;
    double *buf = nullptr; // kSlots x {K, q, out} x kChunk
    cudaStream_t st[kSlots] = {};
};
Staging g_staging[kMaxDevices];

int staging_acquire(Staging &s) {
    if (s.buf)
        return NOA_DCS_SUCCESS;
    cudaError_t e = cudaMalloc((void **)&s.buf, sizeof(double) * 3 * kSlots * kChunk);
    if (e != cudaSuccess) {
        s.buf = nullptr;
        return cuda_fail(e, "cudaMalloc(staging)");
    }
    for (int i = 0; i < kSlots; i++) {
        e = cudaStreamCreateWithFlags(&s.st[i], cudaStreamNonBlocking);
        if (e != cudaSuccess)
            return cuda_fail(e, "cudaStreamCreate");
    }
    return NOA_DCS_SUCCESS;
}

// The device address of a page-locked host buffer of n doubles that the
// kernels can read and write in place (over NVLink-C2C on Grace-Blackwell),
// or nullptr: pageable memory, or a mapping that is not the identity of
// unified addressing.  The first and the last element must both lie in
// page-locked memory.
const double *device_view(const double *p, int64_t n) {
    for (const double *x : {p, p + (n - 1)}) {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, x) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        if (a.type != cudaMemoryTypeHost || a.devicePointer != (const void *)x)
            return nullptr;
    }
    return p;
}

} // namespace

static int vmap_checked(int process, int precision, double *result, const double *K, const double *q, int64_t n,
                        const noa_dcs_element *element, double mass, void *stream, float tol);

extern "C" {

int noa_dcs_cuda_vmap_fp32c(int process, double *result, const double *K, const double *q, int64_t n,
                            const noa_dcs_element *element, double mass, float tolerance, void *stream) {
    if (!(tolerance > 0.f) || !(tolerance < 1.f))
        return fail(NOA_DCS_ERROR_INVALID_VALUE, "FP32C tolerance must lie in (0, 1), got %g", (double)tolerance);
    return vmap_checked(process, NOA_DCS_FP32C, result, K, q, n, element, mass, stream, tolerance);
}

int noa_dcs_cuda_vmap(int process, int precision, double *result, const double *K, const double *q, int64_t n,
                      const noa_dcs_element *element, double mass, void *stream) {
    return vmap_checked(process, precision, result, K, q, n, element, mass, stream, NOA_DCS_FP32C_DEFAULT_TOL);
}

} // extern "C"

static int vmap_checked(int process, int precision, double *result, const double *K, const double *q, int64_t n,
                        const noa_dcs_element *element, double mass, void *stream, float tol) {
    g_last_error[0] = '\0';
    int st = check_common(process, precision, n, mass);
    if (st)
        return st;
    if ((st = check_element(element)))
        return st;
    if (n == 0)
        return NOA_DCS_SUCCESS;
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaGetDevice");
    if ((st = check_device_buffer(result, "result", device)) || (st = check_device_buffer(K, "K", device)) ||
        (st = check_device_buffer(q, "q", device)))
        return st;
    if (overlaps_partially(result, K, n) || overlaps_partially(result, q, n))
        return fail(NOA_DCS_ERROR_OVERLAP, "result partially overlaps an input");
    noa_dcs_consts c;
    noa_dcs_fill_consts(&c, element->A, element->I, element->Z, mass);
    return launch(process, precision, result, K, q, n, &c, (cudaStream_t)stream, tol);
}

extern "C" {

int noa_dcs_cuda_vmap_bremsstrahlung(double *result, const double *K, const double *q, int64_t n,
                                     const noa_dcs_element *element, double mass, void *stream) {
    return noa_dcs_cuda_vmap(NOA_DCS_BREMSSTRAHLUNG, NOA_DCS_FP64, result, K, q, n, element, mass, stream);
}

int noa_dcs_cuda_vmap_pair_production(double *result, const double *K, const double *q, int64_t n,
                                      const noa_dcs_element *element, double mass, void *stream) {
    return noa_dcs_cuda_vmap(NOA_DCS_PAIR_PRODUCTION, NOA_DCS_FP64, result, K, q, n, element, mass, stream);
}

int noa_dcs_cuda_vmap_photonuclear(double *result, const double *K, const double *q, int64_t n,
                                   const noa_dcs_element *element, double mass, void *stream) {
    return noa_dcs_cuda_vmap(NOA_DCS_PHOTONUCLEAR, NOA_DCS_FP64, result, K, q, n, element, mass, stream);
}

int noa_dcs_cuda_vmap_ionisation(double *result, const double *K, const double *q, int64_t n,
                                 const noa_dcs_element *element, double mass, void *stream) {
    return noa_dcs_cuda_vmap(NOA_DCS_IONISATION, NOA_DCS_FP64, result, K, q, n, element, mass, stream);
}

int noa_dcs_cuda_recoil_integral(int process, int moment, double *result, const double *K, int64_t n, double xlow,
                                 const noa_dcs_element *element, double mass, int32_t min_points, void *stream) {
    g_last_error[0] = '\0';
    int st = check_common(process, NOA_DCS_FP64, n, mass);
    if (st)
        return st;
    if ((st = check_element(element)))
        return st;
    if (moment != 0 && moment != 1)
        return fail(NOA_DCS_ERROR_INVALID_VALUE, "moment must be 0 (DEL) or 1 (CEL), got %d", moment);
    if (min_points < 1 || min_points > 1536)
        return fail(NOA_DCS_ERROR_INVALID_VALUE, "min_points must lie in 1..1536, got %d", (int)min_points);
    if (!std::isfinite(xlow) || !(xlow > 0.) || !(xlow <= 1.))
        return fail(NOA_DCS_ERROR_INVALID_VALUE, "xlow must lie in (0, 1], got %g", xlow);
    if (n == 0)
        return NOA_DCS_SUCCESS;
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaGetDevice");
    if ((st = check_device_buffer(result, "result", device)) || (st = check_device_buffer(K, "K", device)))
        return st;
    if (overlaps_partially(result, K, n))
        return fail(NOA_DCS_ERROR_OVERLAP, "result partially overlaps K");
    noa_dcs_consts c;
    noa_dcs_fill_consts(&c, element->A, element->I, element->Z, mass);
    e = noa_dcs_launch_recoil_integral(process, moment, K, result, n, xlow, min_points, &c, (cudaStream_t)stream);
    if (e != cudaSuccess)
        return cuda_fail(e, "recoil integral launch");
    return NOA_DCS_SUCCESS;
}

// ------------------------------------------------- per-K transport functions
namespace {

int current_device(int &device) {
    const cudaError_t e = cudaGetDevice(&device);
    return e == cudaSuccess ? NOA_DCS_SUCCESS : cuda_fail(e, "cudaGetDevice");
}

// Every named buffer must be device memory of the current device.
int check_buffers(std::initializer_list<std::pair<const void *, const char *>> bufs) {
    int device = 0, st;
    if ((st = current_device(device)))
        return st;
    for (const auto &b : bufs)
        if ((st = check_device_buffer(b.first, b.second, device)))
            return st;
    return NOA_DCS_SUCCESS;
}

int check_size_mass(int64_t n, double mass) {
    if (n < 0)
        return fail(NOA_DCS_ERROR_INVALID_VALUE, "negative size %lld", (long long)n);
    if (!std::isfinite(mass) || !(mass > 0.))
        return fail(NOA_DCS_ERROR_INVALID_VALUE, "invalid particle mass %g", mass);
    return NOA_DCS_SUCCESS;
}

} // namespace

int noa_dcs_cuda_soft_scattering(double *result, const double *K, int64_t n, const noa_dcs_element *element,
                                 double mass, void *stream) {
    g_last_error[0] = '\0';
    int st;
    if ((st = check_size_mass(n, mass)) || (st = check_element(element)))
        return st;
    if (n == 0)
        return NOA_DCS_SUCCESS;
    if ((st = check_buffers({{result, "result"}, {K, "K"}})))
        return st;
    if (overlaps_partially(result, K, n))
        return fail(NOA_DCS_ERROR_OVERLAP, "result partially overlaps K");
    noa_dcs_consts c;
    noa_dcs_fill_consts(&c, element->A, element->I, element->Z, mass);
    const cudaError_t e = noa_dcs_launch_soft_scattering(K, result, n, &c, (cudaStream_t)stream);
    return e == cudaSuccess ? NOA_DCS_SUCCESS : cuda_fail(e, "soft scattering launch");
}

int noa_dcs_cuda_coulomb_data(double *fCM, double *screen, double *fspin, double *invlambda, const double *K,
                              int64_t n, const noa_dcs_element *element, double mass, void *stream) {
    g_last_error[0] = '\0';
    int st;
    if ((st = check_size_mass(n, mass)) || (st = check_element(element)))
        return st;
    if (n == 0)
        return NOA_DCS_SUCCESS;
    if ((st = check_buffers({{fCM, "fCM"}, {screen, "screen"}, {fspin, "fspin"}, {invlambda, "invlambda"},
                             {K, "K"}})))
        return st;
    noa_coulomb_element e;
    e.A = element->A;
    e.A13 = std::pow(element->A, 1. / 3);  // dcs.hh:545-546
    e.Z23 = std::pow((double)element->Z, 2. / 3.);  // dcs.hh:589
    e.Z = element->Z;
    const cudaError_t ce = noa_dcs_launch_coulomb_data(K, n, &e, mass, fCM, screen, fspin, invlambda,
                                                       (cudaStream_t)stream);
    return ce == cudaSuccess ? NOA_DCS_SUCCESS : cuda_fail(ce, "coulomb data launch");
}

int noa_dcs_cuda_coulomb_transport(double *coefficients, const double *screen, const double *fspin,
                                   const double *mu, int64_t n_mu, int64_t n, void *stream) {
    g_last_error[0] = '\0';
    if (n < 0)
        return fail(NOA_DCS_ERROR_INVALID_VALUE, "negative size %lld", (long long)n);
    if (n == 0)
        return NOA_DCS_SUCCESS;
    if (n_mu != 1 && n_mu != n)
        return fail(NOA_DCS_ERROR_INVALID_VALUE, "mu must hold 1 or n = %lld values, got %lld", (long long)n,
                    (long long)n_mu);
    int st;
    if ((st = check_buffers({{coefficients, "coefficients"}, {screen, "screen"}, {fspin, "fspin"}, {mu, "mu"}})))
        return st;
    const cudaError_t e =
        noa_dcs_launch_coulomb_transport(screen, fspin, mu, n_mu, n, coefficients, (cudaStream_t)stream);
    return e == cudaSuccess ? NOA_DCS_SUCCESS : cuda_fail(e, "coulomb transport launch");
}

int noa_dcs_cuda_hard_scattering(double *mu0, double *lb_h, const double *G, const double *fCM,
                                 const double *screen, const double *invlambda, const double *fspin, int64_t nel,
                                 int64_t nkin, void *stream) {
    g_last_error[0] = '\0';
    if (nkin < 0 || nel < 1)
        return fail(NOA_DCS_ERROR_INVALID_VALUE, "need nel >= 1 and nkin >= 0, got %lld, %lld", (long long)nel,
                    (long long)nkin);
    if (nkin == 0)
        return NOA_DCS_SUCCESS;
    int st;
    if ((st = check_buffers({{mu0, "mu0"}, {lb_h, "lb_h"}, {G, "G"}, {fCM, "fCM"}, {screen, "screen"},
                             {invlambda, "invlambda"}, {fspin, "fspin"}})))
        return st;
    if (mu0 == lb_h || overlaps_partially(mu0, lb_h, nkin))
        return fail(NOA_DCS_ERROR_OVERLAP, "mu0 and lb_h overlap");
    const double max_mu0 = 0.5 * (1. - std::cos(1E+00 * M_PI / 180.));  // physics.hh:81-84
    const cudaError_t e = noa_dcs_launch_hard_scattering(G, fCM, screen, invlambda, fspin, nel, nkin, max_mu0, mu0,
                                                         lb_h, (cudaStream_t)stream);
    return e == cudaSuccess ? NOA_DCS_SUCCESS : cuda_fail(e, "hard scattering launch");
}

int noa_dcs_vmap_host(int process, int precision, double *result, const double *K, const double *q, int64_t n,
                      const noa_dcs_element *element, double mass) {
    g_last_error[0] = '\0';
    int st = check_common(process, precision, n, mass);
    if (st)
        return st;
    if ((st = check_element(element)))
        return st;
    if (n == 0)
        return NOA_DCS_SUCCESS;
    if (!result || !K || !q)
        return fail(NOA_DCS_ERROR_INVALID_VALUE, "NULL buffer");
    if (overlaps_partially(result, K, n) || overlaps_partially(result, q, n))
        return fail(NOA_DCS_ERROR_OVERLAP, "result partially overlaps an input");
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaGetDevice");
    if (device < 0 || device >= kMaxDevices)
        return fail(NOA_DCS_ERROR_INVALID_VALUE, "device %d out of range", device);
    noa_dcs_consts c;
    noa_dcs_fill_consts(&c, element->A, element->I, element->Z, mass);

    Staging &s = g_staging[device];
    std::lock_guard<std::mutex> lock(s.mu);
    if ((st = staging_acquire(s)))
        return st;
    // page-locked buffers: the kernels read K and q and write the result in
    // place, with no staging copies (the link carries the same 24 bytes per
    // pair, overlapped with the compute by the kernels' own loads and stores)
    if (device_view(K, n) && device_view(q, n) && device_view(result, n)) {
        if ((st = launch(process, precision, result, K, q, n, &c, s.st[0])))
            return st;
        if ((e = cudaStreamSynchronize(s.st[0])) != cudaSuccess)
            return cuda_fail(e, "cudaStreamSynchronize");
        return NOA_DCS_SUCCESS;
    }
    for (int64_t off = 0, chunk = 0; off < n; off += kChunk, chunk++) {
        const int slot = (int)(chunk % kSlots);
        const int64_t m = (n - off) < kChunk ? (n - off) : kChunk;
        double *dK = s.buf + (int64_t)slot * 3 * kChunk;
        double *dQ = dK + kChunk;
        double *dO = dQ + kChunk;
        const size_t bytes = sizeof(double) * (size_t)m;
        if ((e = cudaMemcpyAsync(dK, K + off, bytes, cudaMemcpyDefault, s.st[slot])) != cudaSuccess ||
            (e = cudaMemcpyAsync(dQ, q + off, bytes, cudaMemcpyDefault, s.st[slot])) != cudaSuccess)
            return cuda_fail(e, "cudaMemcpyAsync(host to device)");
        if ((st = launch(process, precision, dO, dK, dQ, m, &c, s.st[slot])))
            return st;
        if ((e = cudaMemcpyAsync(result + off, dO, bytes, cudaMemcpyDefault, s.st[slot])) != cudaSuccess)
            return cuda_fail(e, "cudaMemcpyAsync(device to host)");
    }
    for (int i = 0; i < kSlots; i++)
        if ((e = cudaStreamSynchronize(s.st[i])) != cudaSuccess)
            return cuda_fail(e, "cudaStreamSynchronize");
    return NOA_DCS_SUCCESS;
}

int noa_dcs_release_staging(void) {
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaGetDevice");
    if (device < 0 || device >= kMaxDevices)
        return NOA_DCS_SUCCESS;
    Staging &s = g_staging[device];
    std::lock_guard<std::mutex> lock(s.mu);
    for (int i = 0; i < kSlots; i++)
        if (s.st[i]) {
            cudaStreamSynchronize(s.st[i]);
            cudaStreamDestroy(s.st[i]);
            s.st[i] = nullptr;
        }
    if (s.buf) {
        cudaFree(s.buf);
        s.buf = nullptr;
    }
    return NOA_DCS_SUCCESS;
}

const char *noa_dcs_status_string(int status) {
    switch (status) {
    case NOA_DCS_SUCCESS: return "success";
    case NOA_DCS_ERROR_INVALID_VALUE: return "invalid value";
    case NOA_DCS_ERROR_INVALID_ELEMENT: return "invalid element";
    case NOA_DCS_ERROR_MISALIGNED: return "misaligned buffer";
    case NOA_DCS_ERROR_NOT_DEVICE_MEMORY: return "not device memory";
    case NOA_DCS_ERROR_OVERLAP: return "result partially overlaps an input";
    case NOA_DCS_ERROR_CUDA: return "CUDA error";
    case NOA_DCS_ERROR_TIMEOUT: return "device-side wait timed out";
    case NOA_DCS_ERROR_NOT_SUPPORTED: return "not supported";
    default: return "unknown status";
    }
}

const char *noa_dcs_last_error(void) { return g_last_error; }

int noa_dcs_abi_version(void) { return NOA_DCS_ABI_VERSION; }

} // extern "C"
