/*
 * Python extension mirroring the reference notebook's `muons_cuda` module
 * (docs/pms/muon_dcs.cu:8-16), which exposes the CUDA bremsstrahlung of
 * standard rock for muons.  Here all four processes are exposed (the
 * reference's CPU module docs/pms/muon_dcs.cc:34-44 has the same four names),
 * each calling the LibTorch drop-in noa::pms::dcs::cuda::map_<process>; the
 * element and mass default to STANDARD_ROCK and MUON_MASS as in the notebook
 * and can be overridden.  The GIL is released around each call.
 */
#include "noa_gb300/dcs_cuda.hh"

#include <torch/extension.h>

using namespace noa::pms;

namespace {

AtomicElement element_of(double A, double I, int32_t Z) { return AtomicElement{A, I, Z}; }

} // namespace

PYBIND11_MODULE(_muons_cuda, m) {
    m.def(
        "bremsstrahlung",
        [](torch::Tensor K, torch::Tensor q, double A, double I, int32_t Z, double mass) {
            return dcs::cuda::map_bremsstrahlung(K, q, element_of(A, I, Z), mass);
        },
        py::arg("kinetic_energies"), py::arg("recoil_energies"), py::arg("A") = STANDARD_ROCK.A,
        py::arg("I") = STANDARD_ROCK.I, py::arg("Z") = STANDARD_ROCK.Z, py::arg("mass") = MUON_MASS,
        py::call_guard<py::gil_scoped_release>(), "Bremsstrahlung DCS on CUDA (standard rock, muon by default)");
    m.def(
        "pair_production",
        [](torch::Tensor K, torch::Tensor q, double A, double I, int32_t Z, double mass) {
            return dcs::cuda::map_pair_production(K, q, element_of(A, I, Z), mass);
        },
        py::arg("kinetic_energies"), py::arg("recoil_energies"), py::arg("A") = STANDARD_ROCK.A,
        py::arg("I") = STANDARD_ROCK.I, py::arg("Z") = STANDARD_ROCK.Z, py::arg("mass") = MUON_MASS,
        py::call_guard<py::gil_scoped_release>(), "Pair production DCS on CUDA");
    m.def(
        "photonuclear",
        [](torch::Tensor K, torch::Tensor q, double A, double I, int32_t Z, double mass) {
            return dcs::cuda::map_photonuclear(K, q, element_of(A, I, Z), mass);
        },
        py::arg("kinetic_energies"), py::arg("recoil_energies"), py::arg("A") = STANDARD_ROCK.A,
        py::arg("I") = STANDARD_ROCK.I, py::arg("Z") = STANDARD_ROCK.Z, py::arg("mass") = MUON_MASS,
        py::call_guard<py::gil_scoped_release>(), "Photonuclear DCS on CUDA");
    m.def(
        "ionisation",
        [](torch::Tensor K, torch::Tensor q, double A, double I, int32_t Z, double mass) {
            return dcs::cuda::map_ionisation(K, q, element_of(A, I, Z), mass);
        },
        py::arg("kinetic_energies"), py::arg("recoil_energies"), py::arg("A") = STANDARD_ROCK.A,
        py::arg("I") = STANDARD_ROCK.I, py::arg("Z") = STANDARD_ROCK.Z, py::arg("mass") = MUON_MASS,
        py::call_guard<py::gil_scoped_release>(), "Ionisation DCS on CUDA");
    m.def(
        "vmap",
        [](int process, int precision, torch::Tensor result, torch::Tensor K, torch::Tensor q, double A, double I,
           int32_t Z, double mass) { dcs::cuda::vmap(process, precision, result, K, q, element_of(A, I, Z), mass); },
        py::arg("process"), py::arg("precision"), py::arg("result"), py::arg("kinetic_energies"),
        py::arg("recoil_energies"), py::arg("A") = STANDARD_ROCK.A, py::arg("I") = STANDARD_ROCK.I,
        py::arg("Z") = STANDARD_ROCK.Z, py::arg("mass") = MUON_MASS, py::call_guard<py::gil_scoped_release>(),
        "In-place DCS of one process with a precision selector");
}
