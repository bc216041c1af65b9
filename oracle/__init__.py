"""CPU oracle of the muon DCS path -- TEST INFRASTRUCTURE ONLY.

Python access (ctypes) to oracle/liboracle_dcs.so, the scalar C++
restatement in dcs_oracle.hpp of the reference's src/noa/pms/dcs.hh and
physics.hh, and, where oracle/build_ref.sh built them (from a noa checkout or
its staged headers), to the reference's own code: oracle/_ref/libnoa_ref_dcs.so
(dcs.hh on the CPU), oracle/_ref/libnoa_ref_cuda.so (its CUDA bremsstrahlung
kernel, dcs.cuh) and oracle/_ref/ref_dropin_caller.  Only tests/,
__graft_entry__.smoke() and bench.py's baseline legs may use this package; the
product (noa_gb300) never imports it.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "liboracle_dcs.so")
REF_LIB = os.path.join(HERE, "_ref", "libnoa_ref_dcs.so")              # no FMA contraction: parity build
REF_BENCH_LIB = os.path.join(HERE, "_ref", "libnoa_ref_dcs_bench.so")  # the reference benchmark's flags
REF_CUDA_LIB = os.path.join(HERE, "_ref", "libnoa_ref_cuda.so")
REF_CALLER = os.path.join(HERE, "_ref", "ref_dropin_caller")

_P = ctypes.c_void_p
_D = ctypes.c_double
_I64 = ctypes.c_int64
_I32 = ctypes.c_int32
_INT = ctypes.c_int

_oracle = None
_ref = {}
_ref_cuda = None


def _ptr(a):
    return a.ctypes.data_as(_P)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def lib():
    global _oracle
    if _oracle is None:
        if not os.path.exists(ORACLE_LIB):
            raise RuntimeError(f"{ORACLE_LIB} is not built; run `python -m noa_gb300.build`")
        L = ctypes.CDLL(ORACLE_LIB)
        L.oracle_dcs_vmap.argtypes = [_INT, _P, _P, _P, _I64, _D, _D, _I32, _D, _INT]
        L.oracle_dcs_vmap.restype = _INT
        L.oracle_recoil_integral_vmap.argtypes = [_INT, _INT, _P, _P, _I64, _D, _D, _D, _I32, _D,
                                                  ctypes.c_uint32, _INT]
        L.oracle_recoil_integral_vmap.restype = _INT
        L.oracle_dcs_opcount.argtypes = [_INT, _P, _P, _I64, _D, _D, _I32, _D, _P]
        L.oracle_dcs_opcount.restype = _D
        L.oracle_max_threads.restype = _INT
        _elastic_signatures(L, "oracle")
        L.oracle_soft_scattering.argtypes = [_P, _P, _I64, _D, _D, _I32, _D, _INT]
        L.oracle_soft_scattering.restype = _INT
        _oracle = L
    return _oracle


def _elastic_signatures(L, prefix):
    for name, args in (("coulomb_data", [_P, _I64, _D, _D, _I32, _D, _P, _P, _P, _P]),
                       ("coulomb_transport", [_P, _P, _P, _I64, _I64, _P]),
                       ("hard_scattering", [_P, _P, _P, _P, _P, _I64, _I64, _P, _P])):
        f = getattr(L, f"{prefix}_{name}")
        f.argtypes = args
        f.restype = _INT


def ref_available(build="parity"):
    return os.path.exists(REF_LIB if build == "parity" else REF_BENCH_LIB)


def ref_lib(build="parity"):
    """The compiled reference: build "parity" (-O3, no FMA contraction: bit
    for bit the build that made the goldens) or "bench" (the reference
    benchmark's flags, the compiler's default contraction)."""
    if build not in _ref:
        path = REF_LIB if build == "parity" else REF_BENCH_LIB
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is not built (needs a noa checkout or its staged headers)")
        L = ctypes.CDLL(path)
        L.ref_dcs_vmap.argtypes = [_INT, _INT, _P, _P, _P, _I64, _D, _D, _I32, _D]
        L.ref_dcs_vmap.restype = _INT
        L.ref_recoil_integral_vmap.argtypes = [_INT, _INT, _P, _P, _I64, _D, _D, _D, _I32, _D, _I32]
        L.ref_recoil_integral_vmap.restype = _INT
        _elastic_signatures(L, "ref")
        L.ref_soft_scattering.argtypes = [_P, _P, _I64, _D, _D, _I32, _D]
        L.ref_soft_scattering.restype = _INT
        _ref[build] = L
    return _ref[build]


def ref_cuda_available():
    return os.path.exists(REF_CUDA_LIB)


def ref_cuda_lib():
    """The reference's CUDA bremsstrahlung kernel (dcs.cuh:30-41) behind
    ref_cuda_vmap_bremsstrahlung(result, K, q, n, A, I, Z, mass): device
    pointers of the current device, launched on the legacy default stream."""
    global _ref_cuda
    if _ref_cuda is None:
        if not ref_cuda_available():
            raise RuntimeError(f"{REF_CUDA_LIB} is not built (needs a noa checkout or its staged headers)")
        L = ctypes.CDLL(REF_CUDA_LIB)
        L.ref_cuda_vmap_bremsstrahlung.argtypes = [_P, _P, _P, _I64, _D, _D, _I32, _D]
        L.ref_cuda_vmap_bremsstrahlung.restype = _INT
        _ref_cuda = L
    return _ref_cuda


def ref_cuda_bremsstrahlung(result_ptr, K_ptr, q_ptr, n, element, mass):
    """Enqueues the reference's own CUDA kernel on device buffers (raw
    pointers); raises on a launch error."""
    rc = ref_cuda_lib().ref_cuda_vmap_bremsstrahlung(_P(result_ptr), _P(K_ptr), _P(q_ptr), int(n),
                                                     float(element.A), float(element.I), int(element.Z),
                                                     float(mass))
    if rc:
        raise RuntimeError(f"reference CUDA kernel launch failed ({rc})")


def dcs(process, K, q, element, mass, threads=0):
    """Oracle DCS of one process over arrays K, q.  threads: 0 = all OpenMP
    threads, 1 = the serial loop."""
    K, q = _f64(K), _f64(q)
    out = np.empty_like(K)
    rc = lib().oracle_dcs_vmap(int(process), _ptr(K), _ptr(q), _ptr(out), K.size, float(element.A),
                               float(element.I), int(element.Z), float(mass), int(threads))
    if rc:
        raise ValueError(f"oracle_dcs_vmap failed ({rc})")
    return out


def recoil_integral(process, moment, K, xlow, element, mass, min_points=180, threads=0):
    """Oracle DEL (moment 0) / CEL (moment 1) recoil integral per K."""
    K = _f64(K)
    out = np.empty_like(K)
    rc = lib().oracle_recoil_integral_vmap(int(process), int(moment), _ptr(K), _ptr(out), K.size, float(xlow),
                                           float(element.A), float(element.I), int(element.Z), float(mass),
                                           int(min_points), int(threads))
    if rc:
        raise ValueError(f"oracle_recoil_integral_vmap failed ({rc})")
    return out


def opcount(process, K, q, element, mass):
    """Operation counts {add, mul, div, sqrt, cmp, trans} summed over the pairs."""
    K, q = _f64(K), _f64(q)
    c = np.zeros(6)
    lib().oracle_dcs_opcount(int(process), _ptr(K), _ptr(q), K.size, float(element.A), float(element.I),
                             int(element.Z), float(mass), _ptr(c))
    return dict(zip(("add", "mul", "div", "sqrt", "cmp", "trans"), c.tolist()))


def ref_dcs(process, K, q, element, mass, parallel=False, build="parity"):
    """The reference's own dcs::vmap (or dcs::pvmap) -- only where it was built."""
    K, q = _f64(K), _f64(q)
    out = np.empty_like(K)
    rc = ref_lib(build).ref_dcs_vmap(int(process), int(bool(parallel)), _ptr(K), _ptr(q), _ptr(out), K.size,
                                float(element.A), float(element.I), int(element.Z), float(mass))
    if rc:
        raise ValueError(f"ref_dcs_vmap failed ({rc})")
    return out


def ref_recoil_integral(process, moment, K, xlow, element, mass, min_points=180):
    K = _f64(K)
    out = np.empty_like(K)
    rc = ref_lib().ref_recoil_integral_vmap(int(process), int(moment), _ptr(K), _ptr(out), K.size, float(xlow),
                                            float(element.A), float(element.I), int(element.Z), float(mass),
                                            int(min_points))
    if rc:
        raise ValueError(f"ref_recoil_integral_vmap failed ({rc})")
    return out


def _coulomb_data(L, prefix, K, element, mass):
    K = _f64(K)
    n = K.size
    fCM, screen = np.empty((n, 2)), np.empty((n, 9))
    fspin, invlambda = np.empty(n), np.empty(n)
    getattr(L, f"{prefix}_coulomb_data")(_ptr(K), n, float(element.A), float(element.I), int(element.Z),
                                          float(mass), _ptr(fCM), _ptr(screen), _ptr(fspin), _ptr(invlambda))
    return fCM, screen, fspin, invlambda


def _coulomb_transport(L, prefix, screen, fspin, mu):
    screen, fspin, mu = _f64(screen), _f64(fspin), _f64(np.atleast_1d(mu))
    n = fspin.size
    if mu.size not in (1, n):
        raise ValueError("mu must hold 1 or len(fspin) values")
    coefs = np.empty((n, 2))
    getattr(L, f"{prefix}_coulomb_transport")(_ptr(screen), _ptr(fspin), _ptr(mu), mu.size, n, _ptr(coefs))
    return coefs


def _hard_scattering(L, prefix, G, fCM, screen, invlambda, fspin):
    invlambda = _f64(invlambda)
    if invlambda.ndim == 1:
        invlambda = invlambda[None]
    nel, nkin = invlambda.shape
    G, fCM, screen, fspin = (_f64(a) for a in (G, fCM, screen, fspin))
    if G.size != 2 * nel * nkin or fCM.size != 2 * nel * nkin or screen.size != 9 * nel * nkin \
            or fspin.size != nel * nkin:
        raise ValueError("hard_scattering: inconsistent shapes")
    mu0, lb_h = np.empty(nkin), np.empty(nkin)
    getattr(L, f"{prefix}_hard_scattering")(_ptr(G), _ptr(fCM), _ptr(screen), _ptr(invlambda), _ptr(fspin), nel,
                                            nkin, _ptr(mu0), _ptr(lb_h))
    return mu0, lb_h


def coulomb_data(K, element, mass):
    """Oracle coulomb_data (dcs.hh:604-622): (fCM [n,2], screen [n,9], fspin, invlambda)."""
    return _coulomb_data(lib(), "oracle", K, element, mass)


def coulomb_transport(screen, fspin, mu):
    """Oracle coulomb_transport (dcs.hh:679-699): coefficients [n,2]; mu scalar or [n]."""
    return _coulomb_transport(lib(), "oracle", screen, fspin, mu)


def hard_scattering(G, fCM, screen, invlambda, fspin):
    """Oracle hard_scattering (dcs.hh:840-872) over [nel, nkin] inputs: (mu0, lb_h)."""
    return _hard_scattering(lib(), "oracle", G, fCM, screen, invlambda, fspin)


def soft_scattering(K, element, mass, threads=0):
    """Oracle soft_scattering (dcs.hh:941-952) per K."""
    K = _f64(K)
    out = np.empty_like(K)
    lib().oracle_soft_scattering(_ptr(K), _ptr(out), K.size, float(element.A), float(element.I), int(element.Z),
                                 float(mass), int(threads))
    return out


def ref_coulomb_data(K, element, mass):
    return _coulomb_data(ref_lib(), "ref", K, element, mass)


def ref_coulomb_transport(screen, fspin, mu):
    return _coulomb_transport(ref_lib(), "ref", screen, fspin, mu)


def ref_hard_scattering(G, fCM, screen, invlambda, fspin):
    return _hard_scattering(ref_lib(), "ref", G, fCM, screen, invlambda, fspin)


def ref_soft_scattering(K, element, mass):
    K = _f64(K)
    out = np.empty_like(K)
    ref_lib().ref_soft_scattering(_ptr(K), _ptr(out), K.size, float(element.A), float(element.I), int(element.Z),
                                  float(mass))
    return out


def relative_error(computed, expected):
    """The reference's metric, common.hh:228-236: mean |c - e| / (c + DBL_MIN)."""
    c = np.asarray(computed, dtype=np.float64)
    e = np.asarray(expected, dtype=np.float64)
    return float(np.mean(np.abs((c - e) / (c + np.finfo(np.float64).tiny))))
