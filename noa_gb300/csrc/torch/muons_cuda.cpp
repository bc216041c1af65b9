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
    m.def(
        "recoil_integral",
        [](int process, int moment, torch::Tensor result, torch::Tensor K, double xlow, double A, double I,
           int32_t Z, double mass, int32_t min_points) {
            dcs::cuda::recoil_integral(process, moment, result, K, xlow, element_of(A, I, Z), mass, min_points);
        },
        py::arg("process"), py::arg("moment"), py::arg("result"), py::arg("kinetic_energies"), py::arg("xlow") = 5E-02,
        py::arg("A") = STANDARD_ROCK.A, py::arg("I") = STANDARD_ROCK.I, py::arg("Z") = STANDARD_ROCK.Z,
        py::arg("mass") = MUON_MASS, py::arg("min_points") = 180, py::call_guard<py::gil_scoped_release>(),
        "DEL (moment 0) / CEL (moment 1) recoil integral per kinetic energy, in place");
    m.def(
        "soft_scattering",
        [](torch::Tensor ms1, torch::Tensor K, double A, double I, int32_t Z, double mass) {
            dcs::cuda::soft_scattering(ms1, K, element_of(A, I, Z), mass);
        },
        py::arg("ms1"), py::arg("kinetic_energies"), py::arg("A") = STANDARD_ROCK.A, py::arg("I") = STANDARD_ROCK.I,
        py::arg("Z") = STANDARD_ROCK.Z, py::arg("mass") = MUON_MASS, py::call_guard<py::gil_scoped_release>(),
        "Soft-scattering transverse transport per kinetic energy, in place");
    m.def(
        "coulomb_data",
        [](torch::Tensor fCM, torch::Tensor screening, torch::Tensor fspin, torch::Tensor invlambda, torch::Tensor K,
           double A, double I, int32_t Z, double mass) {
            dcs::cuda::coulomb_data(fCM, screening, fspin, invlambda, K, element_of(A, I, Z), mass);
        },
        py::arg("fCM"), py::arg("screening"), py::arg("fspin"), py::arg("invlambda"), py::arg("kinetic_energies"),
        py::arg("A") = STANDARD_ROCK.A, py::arg("I") = STANDARD_ROCK.I, py::arg("Z") = STANDARD_ROCK.Z,
        py::arg("mass") = MUON_MASS, py::call_guard<py::gil_scoped_release>(), "Elastic scattering data, in place");
    m.def("coulomb_transport", &dcs::cuda::coulomb_transport, py::arg("coefficients"), py::arg("screening"),
          py::arg("fspin"), py::arg("mu"), py::call_guard<py::gil_scoped_release>(),
          "Elastic transport coefficients below the cut-off angle, in place");
    m.def("hard_scattering", &dcs::cuda::hard_scattering, py::arg("mu0"), py::arg("lb_h"), py::arg("coefficients"),
          py::arg("transform"), py::arg("screening"), py::arg("invlambdas"), py::arg("fspins"),
          py::call_guard<py::gil_scoped_release>(), "Hard-scattering cut-off angle and mean free path, in place");
}
