/*
 * LibTorch layer of the drop-in (include/noa_gb300/dcs_cuda.hh): checks the
 * tensors, picks PyTorch's current CUDA stream and calls the C ABI of
 * include/noa_dcs.h.  Mirrors src/noa/pms/dcs.cuh:30-50 of the reference
 * (vmap_* writes result in place; map_* allocates it with zeros_like first).
 */
#include "noa_gb300/dcs_cuda.hh"

#include "noa_dcs.h"

#include <c10/cuda/CUDAGuard.h>
#include <c10/cuda/CUDAStream.h>
#include <torch/torch.h>

namespace noa::pms::dcs::cuda {

namespace {

void check_tensor(const torch::Tensor &t, const char *name, const c10::Device &device) {
    TORCH_CHECK(t.scalar_type() == torch::kFloat64, "expected scalar type Double for ", name, " but found ",
                t.scalar_type());
    TORCH_CHECK(t.is_cuda(), name, " must be a CUDA tensor");
    TORCH_CHECK(t.device() == device, name, " is on ", t.device(), ", expected ", device);
    TORCH_CHECK(t.is_contiguous(), name, " must be contiguous");
}

void run(int process, int precision, const Calculation &result, const Energies &K, const Energies &q,
         const AtomicElement &element, const ParticleMass &mass) {
    TORCH_CHECK(result.defined() && K.defined() && q.defined(), "undefined tensor");
    const c10::Device device = result.device();
    check_tensor(result, "result", device);
    check_tensor(K, "kinetic_energies", device);
    check_tensor(q, "recoil_energies", device);
    const int64_t n = result.numel();
    TORCH_CHECK(K.numel() == n && q.numel() == n, "size mismatch: result ", n, ", kinetic_energies ", K.numel(),
                ", recoil_energies ", q.numel());
    const c10::cuda::CUDAGuard guard(device);
    const noa_dcs_element el{element.A, element.I, element.Z};
    const int st = noa_dcs_cuda_vmap(process, precision, result.data_ptr<double>(), K.data_ptr<double>(),
                                     q.data_ptr<double>(), n, &el, mass,
                                     (void *)c10::cuda::getCurrentCUDAStream(device.index()).stream());
    TORCH_CHECK(st == NOA_DCS_SUCCESS, "noa_dcs: ", noa_dcs_status_string(st), ": ", noa_dcs_last_error());
}

Calculation alloc_and_run(int process, const Energies &K, const Energies &q, const AtomicElement &element,
                          const ParticleMass &mass) {
    const auto result = torch::zeros_like(K);
    run(process, NOA_DCS_FP64, result, K, q, element, mass);
    return result;
}

} // namespace

void vmap(int process, int precision, const Calculation &result, const Energies &kinetic_energies,
          const Energies &recoil_energies, const AtomicElement &element, const ParticleMass &mass) {
    run(process, precision, result, kinetic_energies, recoil_energies, element, mass);
}

#define NOA_DCS_DROP_IN(name, id)                                                                             \
    void vmap_##name(const Calculation &result, const Energies &kinetic_energies,                             \
                     const Energies &recoil_energies, const AtomicElement &element, const ParticleMass &mass) { \
        run(id, NOA_DCS_FP64, result, kinetic_energies, recoil_energies, element, mass);                      \
    }                                                                                                         \
    Calculation map_##name(const Energies &kinetic_energies, const Energies &recoil_energies,                 \
                           const AtomicElement &element, const ParticleMass &mass) {                          \
        return alloc_and_run(id, kinetic_energies, recoil_energies, element, mass);                           \
    }

NOA_DCS_DROP_IN(bremsstrahlung, NOA_DCS_BREMSSTRAHLUNG)
NOA_DCS_DROP_IN(pair_production, NOA_DCS_PAIR_PRODUCTION)
NOA_DCS_DROP_IN(photonuclear, NOA_DCS_PHOTONUCLEAR)
NOA_DCS_DROP_IN(ionisation, NOA_DCS_IONISATION)

#undef NOA_DCS_DROP_IN

} // namespace noa::pms::dcs::cuda
