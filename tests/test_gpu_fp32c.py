"""GPU tests of the FP32-compensated form (NOA_DCS_FP32C) against the FP64
oracle: identical zero pattern, relative error within the tolerance
(1e-6 by default, the accuracy target of the mixed-precision form), and the
explicit-tolerance entry point."""
import ctypes

import numpy as np
import pytest
import torch

import oracle
from noa_gb300 import _lib, dcs
from noa_gb300.elements import ELEMENTS, MUON_MASS, STANDARD_ROCK
from noa_gb300.workload import kinetic_recoil
from tests.parity import PROCESSES, assert_fp64_parity, rel_stats

pytestmark = pytest.mark.gpu

TOL = 1e-6


def fp32c(process, K, q, element=STANDARD_ROCK, mass=MUON_MASS, tol=None):
    tk = torch.from_numpy(np.ascontiguousarray(K)).cuda()
    tq = torch.from_numpy(np.ascontiguousarray(q)).cuda()
    out = torch.full_like(tk, -7.0)
    if tol is None:
        dcs.vmap(process, out, tk, tq, element, mass, precision="fp32c")
    else:
        lib = _lib.load()
        _lib.check(lib.noa_dcs_cuda_vmap_fp32c(process, out.data_ptr(), tk.data_ptr(), tq.data_ptr(), tk.numel(),
                                               _lib.element_struct(element), mass, ctypes.c_float(tol), None))
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
@pytest.mark.parametrize("z", [1, 6, 11, 26, 82])
def test_fp32c_within_tolerance(cuda_device, process, z):
    K, q = kinetic_recoil(1 << 18, offset=5 << 20)
    el = ELEMENTS[z]
    got = fp32c(process, K, q, el)
    exp = oracle.dcs(process, K, q, el, MUON_MASS)
    assert not np.any(got == -7.0)
    s = rel_stats(got, exp)
    print(PROCESSES[process], z, s)
    assert s["zero_agree"] and s["nonfinite_agree"]
    assert s["max"] <= TOL, s
    assert s["median"] <= 1e-7, s


@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
def test_fp32c_golden_and_edges(cuda_device, golden, process):
    for subset in ("seeded", "notebook", "edge"):
        key = f"{subset}_rock_{PROCESSES[process]}"
        got = fp32c(process, golden[f"{subset}_K"], golden[f"{subset}_q"])
        s = rel_stats(got, golden[key])
        assert s["zero_agree"] and s["nonfinite_agree"], (key, s)
        assert s["max"] <= TOL, (key, s)


@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
@pytest.mark.parametrize("tol", [1e-4, 1e-5])
def test_explicit_tolerance(cuda_device, process, tol):
    K, q = kinetic_recoil(1 << 17, offset=9 << 20)
    s = rel_stats(fp32c(process, K, q, tol=tol), oracle.dcs(process, K, q, STANDARD_ROCK, MUON_MASS))
    assert s["zero_agree"] and s["max"] <= tol, s


@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
def test_tiny_tolerance_falls_back_to_fp64(cuda_device, process):
    """A tolerance below float resolution sends every open pair to FP64."""
    K, q = kinetic_recoil(1 << 15, offset=11 << 20)
    assert_fp64_parity(fp32c(process, K, q, tol=1e-12), oracle.dcs(process, K, q, STANDARD_ROCK, MUON_MASS),
                       "fp32c tol=1e-12")


def test_tolerance_argument_checked(cuda_device):
    lib = _lib.load()
    d = torch.zeros(8, dtype=torch.float64, device="cuda")
    el = _lib.element_struct(STANDARD_ROCK)
    for bad in (0.0, -1.0, 1.0, float("nan")):
        assert lib.noa_dcs_cuda_vmap_fp32c(0, d.data_ptr(), d.data_ptr(), d.data_ptr(), 8, el, MUON_MASS,
                                           ctypes.c_float(bad), None) == 1


@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
@pytest.mark.parametrize("n", [1, 31, 257, 1025, 70001])
def test_fp32c_ragged_sizes(cuda_device, process, n):
    K, q = kinetic_recoil(n, offset=123)
    got = fp32c(process, K, q)
    assert not np.any(got == -7.0)
    s = rel_stats(got, oracle.dcs(process, K, q, STANDARD_ROCK, MUON_MASS))
    assert s["zero_agree"] and s["max"] <= TOL


@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
def test_fp32c_large_size(cuda_device, process):
    """1e7 pairs: deterministic, and a 2e5 random sample within tolerance."""
    n = 10_000_000
    K, q = kinetic_recoil(n)
    tk, tq = torch.from_numpy(K).cuda(), torch.from_numpy(q).cuda()
    a = dcs.map(process, tk, tq, precision="fp32c")
    b = dcs.map(process, tk, tq, precision="fp32c")
    torch.cuda.synchronize()
    assert torch.equal(a, b)
    idx = np.random.default_rng(12).choice(n, 200_000, replace=False)
    s = rel_stats(a.cpu().numpy()[idx], oracle.dcs(process, K[idx], q[idx], STANDARD_ROCK, MUON_MASS))
    assert s["zero_agree"] and s["max"] <= TOL, s


@pytest.mark.parametrize("z", sorted(ELEMENTS))
def test_fp32c_pair_production_every_element(cuda_device, z):
    """The pair-production error estimate across all ten elements on 2e6
    pairs each: hydrogen's zeta (comparable to Z, with cancelling numerator
    and denominator) once let a pair through at 1.03e-6."""
    K, q = kinetic_recoil(2_000_000, offset=(50 + z) << 22)
    el = ELEMENTS[z]
    got = fp32c(1, K, q, el)
    exp = oracle.dcs(1, K, q, el, MUON_MASS)
    s = rel_stats(got, exp)
    assert s["zero_agree"] and s["nonfinite_agree"]
    assert s["max"] <= TOL, s


@pytest.mark.parametrize("z", [1, 11, 82])
def test_fp32c_ionisation_bounds(cuda_device, z):
    """Ionisation decides W_max < X K, q > W_max and q <= 0.62 I from a
    float-float W_max with a relative margin of 1e-5, and in FP64 inside it:
    pairs within 1e-16..1e-1 of W_max (both sides), around W_max = X K, at
    0.62 I and across the radiative-correction threshold K = m^2 / (2 me)."""
    rng = np.random.default_rng(40 + z)
    el = ELEMENTS[z] if z != 11 else STANDARD_ROCK
    me, m = 0.510998910e-03, MUON_MASS
    n = 400_000
    K1 = 10 ** rng.uniform(-3, 11, n)
    E = K1 + m
    W = 2 * me * K1 * (K1 + 2 * m) / (m * m + me * (me + 2 * E))
    q1 = W * (1 + rng.choice([-1.0, 1.0], n) * 10 ** rng.uniform(-16, -1, n))
    K2 = 10 ** rng.uniform(-1, 1, n)  # W_max = 0.05 K near K ~ 0.3 GeV
    q2 = K2 * rng.uniform(0.0, 0.06, n)
    wmin = 0.62 * el.I
    K3 = 10 ** rng.uniform(0, 2, n)  # k_rad ~ 10.9 GeV for the muon
    q3 = np.where(rng.random(n) < 0.5, wmin * (1 + rng.integers(-3, 4, n) * 2.0 ** -52), 10 ** rng.uniform(-7, 0, n))
    for K, q in ((K1, q1), (K2, q2), (K3, q3)):
        got = fp32c(3, K, q, el)
        exp = oracle.dcs(3, K, q, el, MUON_MASS)
        s = rel_stats(got, exp)
        assert s["zero_agree"] and s["nonfinite_agree"], s
        assert s["max"] <= TOL, s
