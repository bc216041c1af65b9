"""ctypes binding of the C ABI in include/noa_dcs.h (noa_gb300/libnoa_dcs.so).

There is no fallback: if the library is missing every call raises, telling
the user to build it (`python -m noa_gb300.build`).
"""
import ctypes
import os

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libnoa_dcs.so")

BREMSSTRAHLUNG, PAIR_PRODUCTION, PHOTONUCLEAR, IONISATION = 0, 1, 2, 3
PROCESSES = ("bremsstrahlung", "pair_production", "photonuclear", "ionisation")
FP64, FP32C = 0, 1
PRECISIONS = {"fp64": FP64, "fp32c": FP32C}

SUCCESS = 0
(ERROR_INVALID_VALUE, ERROR_INVALID_ELEMENT, ERROR_MISALIGNED, ERROR_NOT_DEVICE_MEMORY, ERROR_OVERLAP, ERROR_CUDA,
 ERROR_TIMEOUT, ERROR_NOT_SUPPORTED) = range(1, 9)
STATUS_NAMES = {
    0: "NOA_DCS_SUCCESS", 1: "NOA_DCS_ERROR_INVALID_VALUE", 2: "NOA_DCS_ERROR_INVALID_ELEMENT",
    3: "NOA_DCS_ERROR_MISALIGNED", 4: "NOA_DCS_ERROR_NOT_DEVICE_MEMORY", 5: "NOA_DCS_ERROR_OVERLAP",
    6: "NOA_DCS_ERROR_CUDA", 7: "NOA_DCS_ERROR_TIMEOUT", 8: "NOA_DCS_ERROR_NOT_SUPPORTED",
}


class Element(ctypes.Structure):
    """noa_dcs_element: mirrors noa::pms::AtomicElement {A, I, Z} (physics.hh:39-43)."""
    _fields_ = [("A", ctypes.c_double), ("I", ctypes.c_double), ("Z", ctypes.c_int32)]


class DcsError(RuntimeError):
    """A non-zero noa_dcs_status; `.status` holds the code."""

    def __init__(self, status, message):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_D = ctypes.c_double
_INT = ctypes.c_int
_EP = ctypes.POINTER(Element)

# name -> (restype, argtypes); every symbol declared in include/noa_dcs.h.
SIGNATURES = {
    "noa_dcs_cuda_vmap_bremsstrahlung": (_INT, [_P, _P, _P, _I64, _EP, _D, _P]),
    "noa_dcs_cuda_vmap_pair_production": (_INT, [_P, _P, _P, _I64, _EP, _D, _P]),
    "noa_dcs_cuda_vmap_photonuclear": (_INT, [_P, _P, _P, _I64, _EP, _D, _P]),
    "noa_dcs_cuda_vmap_ionisation": (_INT, [_P, _P, _P, _I64, _EP, _D, _P]),
    "noa_dcs_cuda_vmap": (_INT, [_INT, _INT, _P, _P, _P, _I64, _EP, _D, _P]),
    "noa_dcs_cuda_vmap_fp32c": (_INT, [_INT, _P, _P, _P, _I64, _EP, _D, ctypes.c_float, _P]),
    "noa_dcs_vmap_host": (_INT, [_INT, _INT, _P, _P, _P, _I64, _EP, _D]),
    "noa_dcs_cuda_recoil_integral": (_INT, [_INT, _INT, _P, _P, _I64, _D, _EP, _D, ctypes.c_int32, _P]),
    "noa_dcs_cuda_soft_scattering": (_INT, [_P, _P, _I64, _EP, _D, _P]),
    "noa_dcs_cuda_coulomb_data": (_INT, [_P, _P, _P, _P, _P, _I64, _EP, _D, _P]),
    "noa_dcs_cuda_coulomb_transport": (_INT, [_P, _P, _P, _P, _I64, _I64, _P]),
    "noa_dcs_cuda_hard_scattering": (_INT, [_P, _P, _P, _P, _P, _P, _P, _I64, _I64, _P]),
    "noa_dcs_release_staging": (_INT, []),
    "noa_dcs_status_string": (ctypes.c_char_p, [_INT]),
    "noa_dcs_last_error": (ctypes.c_char_p, []),
    "noa_dcs_abi_version": (_INT, []),
    "noa_dcs_batch_plan_create": (_INT, [ctypes.POINTER(_P), _INT, _INT, _INT, _EP, ctypes.POINTER(_I64), _D]),
    "noa_dcs_batch_plan_set_tile": (_INT, [_P, _INT, _INT, _INT]),
    "noa_dcs_batch_plan_get_tile": (_INT, [_P, ctypes.POINTER(_INT), ctypes.POINTER(_INT), ctypes.POINTER(_INT)]),
    "noa_dcs_batch_plan_set_tolerance": (_INT, [_P, ctypes.c_float]),
    "noa_dcs_batch_plan_autotune": (_INT, [_P, _P, _P, _P, _P, _I64]),
    "noa_dcs_batch_plan_execute": (_INT, [_P, _P, _P, _P, _P]),
    "noa_dcs_batch_plan_execute_graph": (_INT, [_P, _P, _P, _P, _P]),
    "noa_dcs_batch_plan_destroy": (_INT, [_P]),
    "noa_dcs_batch_last_error": (ctypes.c_char_p, []),
    "noa_dcs_mlp_create": (_INT, [ctypes.POINTER(_P), _INT, _INT]),
    "noa_dcs_mlp_set_params": (_INT, [_P, _P, _P, _P, _I64, _P]),
    "noa_dcs_mlp_get_params": (_INT, [_P, _P, _P, _P, ctypes.POINTER(_I64)]),
    "noa_dcs_mlp_prepare": (_INT, [_INT, _P, _P, _P, _I64, _EP, _INT, _D, _P, _P, _P, _P]),
    "noa_dcs_mlp_train": (_INT, [_P, _P, _P, _I64, _P, _I64, ctypes.c_float, ctypes.c_float, _P, _P]),
    "noa_dcs_mlp_predict": (_INT, [_P, _P, _P, _I64, _P]),
    "noa_dcs_mlp_gradient": (_INT, [_P, _P, _P, _INT, _P, _P, _P]),
    "noa_dcs_mlp_destroy": (_INT, [_P]),
    "noa_dcs_mlp_last_error": (ctypes.c_char_p, []),
    "noa_dcs_mlp_infer": (_INT, [_P, _P, _INT, _EP, ctypes.POINTER(_I64), _D, _P, _P, _P, ctypes.c_float, _P, _P]),
    "noa_dcs_mlp_infer_last_error": (ctypes.c_char_p, []),
    "noa_dcs_mlp_handles": (_INT, [_P, _P, _P, _P, _P]),
    "noa_dcs_cuda_vmap_batched_noalloc": (_INT, [_INT, _INT, _INT, _EP, ctypes.POINTER(_I64), _D, _P, _P, _P, _P]),
}

# Test and bench instruments, noa_gb300/libnoa_dcs_diag.so (csrc/diag/noa_dcs_diag.h).
DIAG_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libnoa_dcs_diag.so")
DIAG_SIGNATURES = {
    "noa_dcs_probe_fma": (_INT, [_INT, _P, _INT, _INT, ctypes.POINTER(_D), _P]),
    "noa_dcs_lean64_eval": (_INT, [_INT, _P, _P, _P, _I64, _P]),
    "noa_dcs_decision_check": (_INT, [_INT, _P, _P, _P, _I64, _D, _D, ctypes.c_int32, _D, _P]),
}

_lib = None
_diag = None


def load(path=LIB_PATH):
    """Loads the library once and declares every C signature."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is not built; run `python -m noa_gb300.build` "
                           "(the DCS kernels have no CPU fallback)")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def load_diag(path=DIAG_PATH):
    """Loads the test / bench instrument library once."""
    global _diag
    if _diag is not None:
        return _diag
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is not built; run `python -m noa_gb300.build`")
    lib = ctypes.CDLL(path)
    for name, (res, args) in DIAG_SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _diag = lib
    return lib


def check(status):
    if status != SUCCESS:
        raise DcsError(status, load().noa_dcs_last_error().decode())


def element_struct(element):
    return Element(float(element.A), float(element.I), int(element.Z))
