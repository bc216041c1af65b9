/*
 * noa_gb300/dcs_cuda.hh -- C++/LibTorch drop-in for noa::pms::dcs::cuda.
 *
 * Declares, with the reference's namespace, names and signatures, the GPU DCS
 * functions of grinisrit/noa src/noa/pms/dcs.hh:1004-1019 (there:
 * bremsstrahlung only, implemented in src/noa/pms/dcs.cuh:30-50), for all four
 * processes.  A program written against the reference links
 * libnoa_dcs_torch.so instead of compiling dcs.cuh; the mangled names are the
 * same because the argument types are the same (noa::pms::AtomicElement,
 * torch::Tensor, double).
 *
 * If the reference's physics.hh is on the include path it is used for the
 * types; otherwise identical definitions follow (physics.hh:29-52).
 *
 * Behaviour: tensors must be contiguous float64 CUDA tensors of equal numel on
 * one device (the reference checks only the dtype, through data_ptr<double>());
 * violations throw c10::Error like the reference's dtype check.  Work is
 * enqueued on PyTorch's current stream of that device, asynchronously.
 */
#pragma once

#include <torch/types.h>

#include <cstdint>

#if __has_include(<noa/pms/physics.hh>)
#include <noa/pms/physics.hh>
#else
namespace noa::pms {
using Scalar = double;
using Index = int32_t;
using ParticleMass = Scalar;
using AtomicNumber = Index;
using AtomicMass = Scalar;
using MeanExcitation = Scalar;
struct AtomicElement {
    AtomicMass A;
    MeanExcitation I;
    AtomicNumber Z;
};
using Energies = torch::Tensor;
using Calculation = torch::Tensor;
constexpr ParticleMass MUON_MASS = 0.10565839;
constexpr AtomicElement STANDARD_ROCK = AtomicElement{22., 0.1364E-6, 11};
} // namespace noa::pms
#endif

namespace noa::pms::dcs::cuda {

void vmap_bremsstrahlung(const Calculation &result, const Energies &kinetic_energies,
                         const Energies &recoil_energies, const AtomicElement &element, const ParticleMass &mass);
Calculation map_bremsstrahlung(const Energies &kinetic_energies, const Energies &recoil_energies,
                               const AtomicElement &element, const ParticleMass &mass);

void vmap_pair_production(const Calculation &result, const Energies &kinetic_energies,
                          const Energies &recoil_energies, const AtomicElement &element, const ParticleMass &mass);
Calculation map_pair_production(const Energies &kinetic_energies, const Energies &recoil_energies,
                                const AtomicElement &element, const ParticleMass &mass);

void vmap_photonuclear(const Calculation &result, const Energies &kinetic_energies, const Energies &recoil_energies,
                       const AtomicElement &element, const ParticleMass &mass);
Calculation map_photonuclear(const Energies &kinetic_energies, const Energies &recoil_energies,
                             const AtomicElement &element, const ParticleMass &mass);

void vmap_ionisation(const Calculation &result, const Energies &kinetic_energies, const Energies &recoil_energies,
                     const AtomicElement &element, const ParticleMass &mass);
Calculation map_ionisation(const Energies &kinetic_energies, const Energies &recoil_energies,
                           const AtomicElement &element, const ParticleMass &mass);

// Precision-selectable form (no reference counterpart): precision 0 = FP64
// drop-in, 1 = FP32 compensated.
void vmap(int process, int precision, const Calculation &result, const Energies &kinetic_energies,
          const Energies &recoil_energies, const AtomicElement &element, const ParticleMass &mass);

} // namespace noa::pms::dcs::cuda
