"""CPU tests of the FP32C bodies and float-float primitives, built for the
host from the same source as the GPU kernels (noa_gb300/csrc/dcs_fp32c.cuh):
the error estimates bound the error against the oracle, pair production's
float-float screening-log pass takes over the pairs the float form rejects,
and ff_exp / ff_log meet their accuracy.  (The GPU runs of the same checks
are in tests/test_gpu_fp32c.py and tests/test_gpu_lean64.py.)"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import oracle
from noa_gb300.elements import ELEMENTS, MUON_MASS, STANDARD_ROCK
from noa_gb300.workload import kinetic_recoil

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
P = ctypes.c_void_p


@pytest.fixture(scope="module")
def host_lib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("fp32c_host") / "libfp32c_host.so")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off",
                           "-I", os.path.join(ROOT, "noa_gb300", "csrc"),
                           os.path.join(ROOT, "tests", "host", "fp32c_host.cpp"), "-o", out])
    lib = ctypes.CDLL(out)
    lib.fp32c_host_eval.argtypes = [ctypes.c_int, ctypes.c_int, P, P, P, P, ctypes.c_int64, ctypes.c_double,
                                    ctypes.c_double, ctypes.c_int, ctypes.c_double]
    lib.ff_host_eval.argtypes = [ctypes.c_int, P, P, ctypes.c_int64]
    return lib


def evaluate(lib, proc, K, q, el, mode=0):
    K, q = np.ascontiguousarray(K), np.ascontiguousarray(q)
    out = np.empty_like(K)
    est = np.empty(K.size, dtype=np.float32)
    lib.fp32c_host_eval(proc, mode, K.ctypes.data, q.ctypes.data, out.ctypes.data, est.ctypes.data, K.size,
                        el.A, el.I, el.Z, MUON_MASS)
    return out, est


@pytest.mark.parametrize("proc", range(4), ids=["bremsstrahlung", "pair_production", "photonuclear", "ionisation"])
@pytest.mark.parametrize("z", [1, 11, 82])
def test_estimate_bounds_the_error(host_lib, proc, z):
    el = ELEMENTS[z] if z != 11 else STANDARD_ROCK
    K, q = kinetic_recoil(300_000, offset=(70 + z) << 20)
    out, est = evaluate(host_lib, proc, K, q, el)
    ref = oracle.dcs(proc, K, q, el, MUON_MASS)
    nz = ref != 0
    acc = nz & (est <= 1e-6)
    err = np.abs(out[acc] - ref[acc]) / ref[acc]
    assert err.max() < 1e-6, err.max()
    assert np.array_equal(out[~nz & (est <= 1e-6)], ref[~nz & (est <= 1e-6)])  # zeros stay zeros
    assert acc.sum() > 0.9 * nz.sum()


@pytest.mark.parametrize("z", [1, 11, 82])
def test_pair_production_float_float_pass(host_lib, z):
    """The float form rejects ~4% of the open pairs (its screening log Le is
    small there); the float-float pass accepts almost all of them within the
    tolerance, leaving ~0.05% for FP64."""
    el = ELEMENTS[z] if z != 11 else STANDARD_ROCK
    K, q = kinetic_recoil(600_000, offset=(90 + z) << 20)
    ref = oracle.dcs(1, K, q, el, MUON_MASS)
    o1, e1 = evaluate(host_lib, 1, K, q, el, 0)
    o2, e2 = evaluate(host_lib, 1, K, q, el, 1)
    nz = ref != 0
    rejected = nz & ~(e1 <= 1e-6)
    second = rejected & (e2 <= 1e-6)
    assert rejected.sum() > 0.02 * nz.sum()
    assert second.sum() > 0.95 * rejected.sum()
    err = np.abs(o2[second] - ref[second]) / ref[second]
    assert err.max() < 1e-6, err.max()


def test_ionisation_bounds_host(host_lib):
    rng = np.random.default_rng(3)
    me, m = 0.510998910e-03, MUON_MASS
    K = 10 ** rng.uniform(-3, 11, 300_000)
    W = 2 * me * K * (K + 2 * m) / (m * m + me * (me + 2 * (K + m)))
    q = W * (1 + rng.choice([-1.0, 1.0], K.size) * 10 ** rng.uniform(-16, -1, K.size))
    out, est = evaluate(host_lib, 3, K, q, STANDARD_ROCK)
    ref = oracle.dcs(3, K, q, STANDARD_ROCK, MUON_MASS)
    acc = est <= 1e-6
    assert np.array_equal(out[acc] == 0, ref[acc] == 0)
    nz = acc & (ref != 0)
    assert (np.abs(out[nz] - ref[nz]) / ref[nz]).max() < 1e-6


def test_float_float_exp_log(host_lib):
    rng = np.random.default_rng(5)

    def pair(x):
        h = x.astype(np.float32)
        return h.astype(np.longdouble) + (x - h.astype(np.float64)).astype(np.float32).astype(np.longdouble)

    x = np.concatenate([rng.uniform(-70, 80, 100000), rng.uniform(-1e-3, 1e-3, 20000)])
    out = np.empty_like(x)
    host_lib.ff_host_eval(0, x.ctypes.data, out.ctypes.data, x.size)
    ref = np.exp(pair(x))
    assert (np.abs((out.astype(np.longdouble) - ref) / ref)).astype(np.float64).max() <= 5e-13
    x = np.concatenate([np.exp(rng.uniform(np.log(1e-30), np.log(1e30), 100000)), 1 + rng.uniform(-1e-3, 1e-3, 20000)])
    out = np.empty_like(x)
    host_lib.ff_host_eval(1, x.ctypes.data, out.ctypes.data, x.size)
    ref = np.log(pair(x))
    err = np.abs(out.astype(np.longdouble) - ref).astype(np.float64)
    big = np.abs(ref) > 0.1
    assert (err[big] / np.abs(ref[big]).astype(np.float64)).max() <= 5e-13
    assert err[~big].max() <= 3e-14


def test_pair_production_estimate_near_the_recalibration_pair(host_lib):
    """A standard-rock pair near K = 0.74 GeV, q = 0.55 GeV (just below the
    upper bound q = K + m (1 - 0.75 sqrt(e) Z^1/3) ~ K - 0.185 GeV, the
    electron screening term clamped, the muon screening log ~0.28) was once
    accepted by the float form at an error of 1.06e-6: the muon screening
    log's absolute float error reaches ~4 u there.  On 1.2e6 pairs packed
    around it (K and q/K within 5%, and 2e5 of them within 1e-3), plus 1e6
    pairs at q/K ~ 0.68 where most are accepted, the estimate bounds every
    open pair's error, and no accepted pair exceeds the 1e-6 tolerance, in
    the float and the float-float form.  (Errors there reach ~1.3e-6, so the
    pairs nearest the point must be, and are, rejected.)"""
    rng = np.random.default_rng(74)
    nu0 = 0.55 / 0.74
    K = np.concatenate([0.74 * (1 + rng.uniform(-0.05, 0.05, 1_000_000)),
                        0.74 * (1 + rng.uniform(-1e-3, 1e-3, 200_000)),
                        0.74 * (1 + rng.uniform(-0.05, 0.05, 1_000_000))])
    nu = np.concatenate([nu0 * (1 + rng.uniform(-0.05, 0.05, 1_000_000)),
                         nu0 * (1 + rng.uniform(-1e-3, 1e-3, 200_000)),
                         0.5 / 0.74 * (1 + rng.uniform(-0.05, 0.05, 1_000_000))])
    q = nu * K
    ref = oracle.dcs(1, K, q, STANDARD_ROCK, MUON_MASS)
    nz = ref != 0
    assert nz.sum() > 1_500_000
    for mode in (0, 1):
        out, est = evaluate(host_lib, 1, K, q, STANDARD_ROCK, mode)
        err = np.abs(out[nz] - ref[nz]) / ref[nz]
        assert np.all(err < est[nz]), (mode, float((err / est[nz]).max()))
        acc = est[nz] <= 1e-6
        assert acc.sum() > 500_000
        assert err[acc].max() < 1e-6, (mode, float(err[acc].max()))
