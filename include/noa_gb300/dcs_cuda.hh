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
using Energy = Scalar;
constexpr ParticleMass MUON_MASS = 0.10565839;
constexpr AtomicElement STANDARD_ROCK = AtomicElement{22., 0.1364E-6, 11};
namespace dcs {
using InvLambdas = torch::Tensor;
using ScreeningFactors = torch::Tensor;
using FSpins = torch::Tensor;
using CMLorentz = torch::Tensor;
using AngularCutoff = torch::Tensor;
using HSMeanFreePath = torch::Tensor;
using TransportCoefs = torch::Tensor;
} // namespace dcs
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


// GPU forms of the reference's per-K CPU functions (dcs.hh:89-130, 499-952),
// same argument order; every tensor a contiguous float64 CUDA tensor.

// dcs::vmap_integral(dcs::recoil_integral(dcs::<process>, del_integrand |
// cel_integrand))(result, kinetic_energies, xlow, element, mass, min_points):
// process 0..3 as in vmap, moment 0 = DEL, 1 = CEL.
void recoil_integral(int process, int moment, const Calculation &result, const Energies &kinetic_energies,
                     const Energy &xlow, const AtomicElement &element, const AtomicMass &mass, Index min_points);

// dcs::soft_scattering(ms1, kinetic_energies, element, mass), dcs.hh:941-952.
void soft_scattering(const Calculation &ms1, const Energies &kinetic_energies, const AtomicElement &element,
                     const ParticleMass &mass);

// dcs::coulomb_data, dcs.hh:600-622: fCM [n, 2], screening [n, 9], fspin [n], invlambda [n].
void coulomb_data(const CMLorentz &fCM, const ScreeningFactors &screening, const FSpins &fspin,
                  const InvLambdas &invlambda, const Energies &kinetic_energies, const AtomicElement &element,
                  const ParticleMass &mass);

// dcs::coulomb_transport, dcs.hh:674-699: coefficients [n, 2]; mu one value or [n].
void coulomb_transport(const TransportCoefs &coefficients, const ScreeningFactors &screening, const FSpins &fspin,
                       const AngularCutoff &mu);

// dcs::hard_scattering, dcs.hh:842-872: invlambdas / fspins [nel, nkin],
// coefficients / transform [nel, nkin, 2], screening [nel, nkin, 9].
void hard_scattering(const AngularCutoff &mu0, const HSMeanFreePath &lb_h, const TransportCoefs &coefficients,
                     const CMLorentz &transform, const ScreeningFactors &screening, const InvLambdas &invlambdas,
                     const FSpins &fspins);
} // namespace noa::pms::dcs::cuda
