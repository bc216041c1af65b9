"""Python mirror of the reference's GPU DCS surface, noa::pms::dcs::cuda.

Reference: src/noa/pms/dcs.hh:1004-1019 (declarations) and
src/noa/pms/dcs.cuh:30-50 (bremsstrahlung only).  Here all four processes
exist, with the reference's argument order (result, kinetic_energies,
recoil_energies, element, mass) and `map_*` twins that allocate the result
with zeros_like, as dcs.cuh:43-50 does.  Work is enqueued on PyTorch's current
CUDA stream without synchronising.

Argument errors raise RuntimeError, as the reference's data_ptr<double>()
dtype check raises c10::Error; unlike the reference, size, device and
contiguity are checked too (the reference reads out of bounds or silently
misreads on those).
"""
import torch

from . import _lib
from .elements import MUON_MASS, STANDARD_ROCK, X_FRACTION, AtomicElement

__all__ = [
    "vmap", "map", "vmap_host", "recoil_integral", "soft_scattering",
    "coulomb_data", "coulomb_transport", "hard_scattering",
    "vmap_bremsstrahlung", "vmap_pair_production", "vmap_photonuclear", "vmap_ionisation",
    "map_bremsstrahlung", "map_pair_production", "map_photonuclear", "map_ionisation",
]


def _check_tensor(t, name, device=None):
    if not isinstance(t, torch.Tensor):
        raise RuntimeError(f"{name} must be a torch.Tensor")
    if t.dtype != torch.float64:
        raise RuntimeError(f"expected scalar type Double for {name} but found {t.dtype}")
    if not t.is_cuda:
        raise RuntimeError(f"{name} must be a CUDA tensor")
    if device is not None and t.device != device:
        raise RuntimeError(f"{name} is on {t.device}, expected {device}")
    if not t.is_contiguous():
        raise RuntimeError(f"{name} must be contiguous")


def _process_id(process):
    if isinstance(process, str):
        return _lib.PROCESSES.index(process)
    return int(process)


def vmap(process, result, kinetic_energies, recoil_energies, element=STANDARD_ROCK, mass=MUON_MASS,
         precision="fp64"):
    """result[i] = DCS(kinetic_energies[i], recoil_energies[i]) for one process."""
    lib = _lib.load()
    _check_tensor(result, "result")
    _check_tensor(kinetic_energies, "kinetic_energies", result.device)
    _check_tensor(recoil_energies, "recoil_energies", result.device)
    n = result.numel()
    if kinetic_energies.numel() != n or recoil_energies.numel() != n:
        raise RuntimeError(f"size mismatch: result {n}, kinetic_energies {kinetic_energies.numel()}, "
                           f"recoil_energies {recoil_energies.numel()}")
    el = _lib.element_struct(element)
    with torch.cuda.device(result.device):
        stream = torch.cuda.current_stream(result.device).cuda_stream
        _lib.check(lib.noa_dcs_cuda_vmap(_process_id(process), _lib.PRECISIONS[precision],
                                         result.data_ptr(), kinetic_energies.data_ptr(),
                                         recoil_energies.data_ptr(), n, el, float(mass), stream))
    return result


def map(process, kinetic_energies, recoil_energies, element=STANDARD_ROCK, mass=MUON_MASS, precision="fp64"):
    """Allocating twin of vmap (dcs.cuh:43-50)."""
    result = torch.zeros_like(kinetic_energies)
    return vmap(process, result, kinetic_energies, recoil_energies, element, mass, precision)


def vmap_host(process, result, kinetic_energies, recoil_energies, element=STANDARD_ROCK, mass=MUON_MASS,
              precision="fp64"):
    """Host-buffer path (noa_dcs_vmap_host): CPU float64 tensors in and out,
    computed on the GPU; returns when result is filled.  Pinned tensors
    (pin_memory) are read and written in place by the kernels; pageable ones
    are staged through device buffers."""
    lib = _lib.load()
    for t, name in ((result, "result"), (kinetic_energies, "kinetic_energies"),
                    (recoil_energies, "recoil_energies")):
        if t.dtype != torch.float64 or t.is_cuda or not t.is_contiguous():
            raise RuntimeError(f"{name} must be a contiguous float64 CPU tensor")
    n = result.numel()
    if kinetic_energies.numel() != n or recoil_energies.numel() != n:
        raise RuntimeError("size mismatch")
    el = _lib.element_struct(element)
    _lib.check(lib.noa_dcs_vmap_host(_process_id(process), _lib.PRECISIONS[precision], result.data_ptr(),
                                     kinetic_energies.data_ptr(), recoil_energies.data_ptr(), n, el,
                                     float(mass)))
    return result


def recoil_integral(process, moment, result, kinetic_energies, xlow=X_FRACTION, element=STANDARD_ROCK,
                    mass=MUON_MASS, min_points=180):
    """GPU form of dcs::vmap_integral(dcs::recoil_integral(dcs::<process>,
    del_integrand | cel_integrand)) (dcs.hh:89-130): result[i] = the DEL
    (moment 0) or CEL (moment 1) integral for kinetic_energies[i]."""
    lib = _lib.load()
    _check_tensor(result, "result")
    _check_tensor(kinetic_energies, "kinetic_energies", result.device)
    n = result.numel()
    if kinetic_energies.numel() != n:
        raise RuntimeError("size mismatch")
    if isinstance(moment, str):
        moment = {"del": 0, "cel": 1}[moment.lower()]
    el = _lib.element_struct(element)
    with torch.cuda.device(result.device):
        stream = torch.cuda.current_stream(result.device).cuda_stream
        _lib.check(lib.noa_dcs_cuda_recoil_integral(_process_id(process), int(moment), result.data_ptr(),
                                                    kinetic_energies.data_ptr(), n, float(xlow), el, float(mass),
                                                    int(min_points), stream))
    return result


def _stream(t):
    return torch.cuda.current_stream(t.device).cuda_stream


def soft_scattering(ms1, kinetic_energies, element=STANDARD_ROCK, mass=MUON_MASS):
    """GPU form of dcs::soft_scattering (dcs.hh:941-952): ms1[i] = the
    transverse-transport coefficient of ionisation + photonuclear at
    kinetic_energies[i]."""
    lib = _lib.load()
    _check_tensor(ms1, "ms1")
    _check_tensor(kinetic_energies, "kinetic_energies", ms1.device)
    n = ms1.numel()
    if kinetic_energies.numel() != n:
        raise RuntimeError("size mismatch")
    with torch.cuda.device(ms1.device):
        _lib.check(lib.noa_dcs_cuda_soft_scattering(ms1.data_ptr(), kinetic_energies.data_ptr(), n,
                                                    _lib.element_struct(element), float(mass), _stream(ms1)))
    return ms1


def coulomb_data(fCM, screening, fspin, invlambda, kinetic_energies, element=STANDARD_ROCK, mass=MUON_MASS):
    """GPU form of dcs::coulomb_data (dcs.hh:604-622), same argument order:
    fills fCM [n, 2], screening [n, 9], fspin [n] and invlambda [n]."""
    lib = _lib.load()
    _check_tensor(kinetic_energies, "kinetic_energies")
    dev = kinetic_energies.device
    n = kinetic_energies.numel()
    for t, name, width in ((fCM, "fCM", 2), (screening, "screening", 9), (fspin, "fspin", 1),
                           (invlambda, "invlambda", 1)):
        _check_tensor(t, name, dev)
        if t.numel() != width * n:
            raise RuntimeError(f"{name} must hold {width} x {n} values")
    with torch.cuda.device(dev):
        _lib.check(lib.noa_dcs_cuda_coulomb_data(fCM.data_ptr(), screening.data_ptr(), fspin.data_ptr(),
                                                 invlambda.data_ptr(), kinetic_energies.data_ptr(), n,
                                                 _lib.element_struct(element), float(mass), _stream(fCM)))


def coulomb_transport(coefficients, screening, fspin, mu):
    """GPU form of dcs::coulomb_transport (dcs.hh:679-699): coefficients
    [n, 2] below the cut-off angle mu (one value, or one per energy)."""
    lib = _lib.load()
    _check_tensor(fspin, "fspin")
    dev = fspin.device
    n = fspin.numel()
    _check_tensor(coefficients, "coefficients", dev)
    _check_tensor(screening, "screening", dev)
    _check_tensor(mu, "mu", dev)
    if coefficients.numel() != 2 * n or screening.numel() != 9 * n or mu.numel() not in (1, n):
        raise RuntimeError("size mismatch")
    with torch.cuda.device(dev):
        _lib.check(lib.noa_dcs_cuda_coulomb_transport(coefficients.data_ptr(), screening.data_ptr(),
                                                      fspin.data_ptr(), mu.data_ptr(), mu.numel(), n,
                                                      _stream(fspin)))


def hard_scattering(mu0, lb_h, coefficients, transform, screening, invlambdas, fspins):
    """GPU form of dcs::hard_scattering (dcs.hh:840-872), same argument
    order: mu0 and lb_h [nkin] from per-element inputs shaped like the
    reference's, invlambdas and fspins [nel, nkin], coefficients and
    transform [nel, nkin, 2], screening [nel, nkin, 9]."""
    lib = _lib.load()
    _check_tensor(invlambdas, "invlambdas")
    dev = invlambdas.device
    if invlambdas.dim() != 2:
        raise RuntimeError("invlambdas must be [nel, nkin]")
    nel, nkin = invlambdas.shape
    for t, name, width in ((mu0, "mu0", 1), (lb_h, "lb_h", 1), (coefficients, "coefficients", 2 * nel),
                           (transform, "transform", 2 * nel), (screening, "screening", 9 * nel),
                           (fspins, "fspins", nel)):
        _check_tensor(t, name, dev)
        if t.numel() != width * nkin:
            raise RuntimeError(f"{name} must hold {width} x {nkin} values")
    with torch.cuda.device(dev):
        _lib.check(lib.noa_dcs_cuda_hard_scattering(mu0.data_ptr(), lb_h.data_ptr(), coefficients.data_ptr(),
                                                    transform.data_ptr(), screening.data_ptr(),
                                                    invlambdas.data_ptr(), fspins.data_ptr(), nel, nkin,
                                                    _stream(mu0)))


def _bind(pid):
    def _vmap(result, kinetic_energies, recoil_energies, element=STANDARD_ROCK, mass=MUON_MASS):
        return vmap(pid, result, kinetic_energies, recoil_energies, element, mass)

    def _map(kinetic_energies, recoil_energies, element=STANDARD_ROCK, mass=MUON_MASS):
        return map(pid, kinetic_energies, recoil_energies, element, mass)
    return _vmap, _map


vmap_bremsstrahlung, map_bremsstrahlung = _bind(_lib.BREMSSTRAHLUNG)
vmap_pair_production, map_pair_production = _bind(_lib.PAIR_PRODUCTION)
vmap_photonuclear, map_photonuclear = _bind(_lib.PHOTONUCLEAR)
vmap_ionisation, map_ionisation = _bind(_lib.IONISATION)
