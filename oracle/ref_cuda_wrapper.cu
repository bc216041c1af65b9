/*
 * Thin C wrapper around the UNMODIFIED reference CUDA kernel of grinisrit/noa
 * -- BENCHMARK AND TEST INFRASTRUCTURE ONLY.
 *
 * src/noa/pms/dcs.cuh:30-41 defines noa::pms::dcs::cuda::vmap_bremsstrahlung,
 * the reference's only GPU code: a device lambda over _bremsstrahlung_
 * (physics.hh:109-153) launched one thread per pair by
 * utils::cuda::launch_kernel on the legacy default stream
 * (src/noa/utils/common.cuh:39-56).  Compiled by oracle/build_ref.sh for
 * sm_103a with the reference's CUDA flags into oracle/_ref/libnoa_ref_cuda.so,
 * so that it can be timed and checked beside this repository's kernels on the
 * same device buffers.
 */
#include <noa/pms/dcs.cuh>

#include <torch/torch.h>

#include <cuda_runtime.h>

#include <cstdint>

extern "C" {

// result[i] = bremsstrahlung(K[i], q[i]) for i < n, all three device pointers
// of the current device.  Enqueued on the legacy default stream like the
// reference; returns the launch status (cudaGetLastError) as an int.
int ref_cuda_vmap_bremsstrahlung(double *result, const double *K, const double *q, int64_t n, double A, double I,
                                 int32_t Z, double mass) {
    int dev = 0;
    cudaGetDevice(&dev);
    const auto opt = torch::TensorOptions().dtype(torch::kFloat64).device(torch::kCUDA, dev);
    const auto tk = torch::from_blob(const_cast<double *>(K), {n}, opt);
    const auto tq = torch::from_blob(const_cast<double *>(q), {n}, opt);
    const auto tr = torch::from_blob(result, {n}, opt);
    noa::pms::dcs::cuda::vmap_bremsstrahlung(tr, tk, tq, noa::pms::AtomicElement{A, I, Z}, mass);
    return static_cast<int>(cudaGetLastError());
}

} // extern "C"
