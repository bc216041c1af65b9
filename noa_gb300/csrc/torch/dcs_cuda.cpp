/*
 * LibTorch layer of the drop-in (include/noa_gb300/dcs_cuda.hh): checks the
 * tensors, picks PyTorch's current CUDA stream and calls the C ABI of
 * include/noa_dcs.h.  Mirrors src/noa/pms/dcs.cuh:30-50 of the reference
 * (vmap_* writes result in place; map_* allocates it with zeros_like first),
 * and gives GPU forms of the per-K functions of dcs.hh:89-130 and 499-952
 * with the reference's argument lists.
 */
#include "noa_gb300/dcs_cuda.hh"

#include "noa_dcs.h"

#include <c10/cuda/CUDAGuard.h>
#include <c10/cuda/CUDAStream.h>
#include <torch/torch.h>

#include <utility>

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

namespace {

void check_status(int st) {
    TORCH_CHECK(st == NOA_DCS_SUCCESS, "noa_dcs: ", noa_dcs_status_string(st), ": ", noa_dcs_last_error());
}

void check_numel(const torch::Tensor &t, const char *name, int64_t n) {
    TORCH_CHECK(t.defined(), name, " is undefined");
    TORCH_CHECK(t.numel() == n, name, " must hold ", n, " values, has ", t.numel());
}

void *stream_of(const c10::Device &device) {
    return (void *)c10::cuda::getCurrentCUDAStream(device.index()).stream();
}

} // namespace

void recoil_integral(int process, int moment, const Calculation &result, const Energies &kinetic_energies,
                     const Energy &xlow, const AtomicElement &element, const AtomicMass &mass, Index min_points) {
    TORCH_CHECK(result.defined() && kinetic_energies.defined(), "undefined tensor");
    const c10::Device device = result.device();
    check_tensor(result, "result", device);
    check_tensor(kinetic_energies, "kinetic_energies", device);
    check_numel(kinetic_energies, "kinetic_energies", result.numel());
    const c10::cuda::CUDAGuard guard(device);
    const noa_dcs_element el{element.A, element.I, element.Z};
    check_status(noa_dcs_cuda_recoil_integral(process, moment, result.data_ptr<double>(),
                                              kinetic_energies.data_ptr<double>(), result.numel(), xlow, &el, mass,
                                              min_points, stream_of(device)));
}

void soft_scattering(const Calculation &ms1, const Energies &kinetic_energies, const AtomicElement &element,
                     const ParticleMass &mass) {
    TORCH_CHECK(ms1.defined() && kinetic_energies.defined(), "undefined tensor");
    const c10::Device device = ms1.device();
    check_tensor(ms1, "ms1", device);
    check_tensor(kinetic_energies, "kinetic_energies", device);
    check_numel(kinetic_energies, "kinetic_energies", ms1.numel());
    const c10::cuda::CUDAGuard guard(device);
    const noa_dcs_element el{element.A, element.I, element.Z};
    check_status(noa_dcs_cuda_soft_scattering(ms1.data_ptr<double>(), kinetic_energies.data_ptr<double>(),
                                              ms1.numel(), &el, mass, stream_of(device)));
}

void coulomb_data(const CMLorentz &fCM, const ScreeningFactors &screening, const FSpins &fspin,
                  const InvLambdas &invlambda, const Energies &kinetic_energies, const AtomicElement &element,
                  const ParticleMass &mass) {
    TORCH_CHECK(kinetic_energies.defined(), "undefined tensor");
    const c10::Device device = kinetic_energies.device();
    const int64_t n = kinetic_energies.numel();
    check_tensor(kinetic_energies, "kinetic_energies", device);
    check_numel(fCM, "fCM", 2 * n);
    check_numel(screening, "screening", 9 * n);
    check_numel(fspin, "fspin", n);
    check_numel(invlambda, "invlambda", n);
    check_tensor(fCM, "fCM", device);
    check_tensor(screening, "screening", device);
    check_tensor(fspin, "fspin", device);
    check_tensor(invlambda, "invlambda", device);
    const c10::cuda::CUDAGuard guard(device);
    const noa_dcs_element el{element.A, element.I, element.Z};
    check_status(noa_dcs_cuda_coulomb_data(fCM.data_ptr<double>(), screening.data_ptr<double>(),
                                           fspin.data_ptr<double>(), invlambda.data_ptr<double>(),
                                           kinetic_energies.data_ptr<double>(), n, &el, mass, stream_of(device)));
}

void coulomb_transport(const TransportCoefs &coefficients, const ScreeningFactors &screening, const FSpins &fspin,
                       const AngularCutoff &mu) {
    TORCH_CHECK(fspin.defined() && mu.defined(), "undefined tensor");
    const c10::Device device = fspin.device();
    const int64_t n = fspin.numel();
    check_tensor(fspin, "fspin", device);
    check_numel(coefficients, "coefficients", 2 * n);
    check_numel(screening, "screening", 9 * n);
    check_tensor(coefficients, "coefficients", device);
    check_tensor(screening, "screening", device);
    check_tensor(mu, "mu", device);
    TORCH_CHECK(mu.numel() == 1 || mu.numel() == n, "mu must hold 1 or ", n, " values");
    const c10::cuda::CUDAGuard guard(device);
    check_status(noa_dcs_cuda_coulomb_transport(coefficients.data_ptr<double>(), screening.data_ptr<double>(),
                                                fspin.data_ptr<double>(), mu.data_ptr<double>(), mu.numel(), n,
                                                stream_of(device)));
}

void hard_scattering(const AngularCutoff &mu0, const HSMeanFreePath &lb_h, const TransportCoefs &coefficients,
                     const CMLorentz &transform, const ScreeningFactors &screening, const InvLambdas &invlambdas,
                     const FSpins &fspins) {
    TORCH_CHECK(invlambdas.defined() && invlambdas.dim() == 2, "invlambdas must be [nel, nkin]");
    const c10::Device device = invlambdas.device();
    const int64_t nel = invlambdas.size(0), nkin = invlambdas.size(1);
    check_numel(mu0, "mu0", nkin);
    check_numel(lb_h, "lb_h", nkin);
    check_numel(coefficients, "coefficients", 2 * nel * nkin);
    check_numel(transform, "transform", 2 * nel * nkin);
    check_numel(screening, "screening", 9 * nel * nkin);
    check_numel(fspins, "fspins", nel * nkin);
    for (const auto &[t, name] : {std::pair<const torch::Tensor &, const char *>{mu0, "mu0"}, {lb_h, "lb_h"},
                                  {coefficients, "coefficients"}, {transform, "transform"},
                                  {screening, "screening"}, {invlambdas, "invlambdas"}, {fspins, "fspins"}})
        check_tensor(t, name, device);
    const c10::cuda::CUDAGuard guard(device);
    check_status(noa_dcs_cuda_hard_scattering(mu0.data_ptr<double>(), lb_h.data_ptr<double>(),
                                              coefficients.data_ptr<double>(), transform.data_ptr<double>(),
                                              screening.data_ptr<double>(), invlambdas.data_ptr<double>(),
                                              fspins.data_ptr<double>(), nel, nkin, stream_of(device)));
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
