"""CPU tests of the C ABI: the library loads, exports every symbol that
include/noa_dcs.h declares, and rejects bad arguments before touching CUDA
(so these run without a GPU)."""
import ctypes
import os
import re

import pytest

from noa_gb300 import _lib
from noa_gb300.elements import MUON_MASS, STANDARD_ROCK

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "noa_dcs.h")


def declared_functions(path=HEADER):
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(noa_dcs_\w+)\s*\(", text)))


def test_header_declares_the_bound_signatures():
    assert declared_functions() == sorted(_lib.SIGNATURES)


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(_lib.LIB_PATH)
    missing = [f for f in declared_functions() if not hasattr(lib, f)]
    assert not missing


DIAG_HEADER = os.path.join(os.path.dirname(HEADER), os.pardir, "noa_gb300", "csrc", "diag", "noa_dcs_diag.h")


def test_instruments_live_outside_the_product_library(built):
    """The FMA probe and the function evaluator are declared in the
    instrument header and exported by libnoa_dcs_diag.so only."""
    diag = declared_functions(DIAG_HEADER)
    assert diag == sorted(_lib.DIAG_SIGNATURES)
    assert not set(diag) & set(declared_functions())
    product = ctypes.CDLL(_lib.LIB_PATH)
    assert not any(hasattr(product, f) for f in diag)
    inst = ctypes.CDLL(_lib.DIAG_PATH)
    assert all(hasattr(inst, f) for f in diag)


def test_abi_version_and_status_strings(built):
    lib = _lib.load()
    assert lib.noa_dcs_abi_version() == 1
    for code in range(9):
        assert lib.noa_dcs_status_string(code).decode()
    assert lib.noa_dcs_status_string(99).decode() == "unknown status"


def test_element_struct_layout():
    # noa::pms::AtomicElement {double A; double I; int32_t Z;}: 24 bytes, Z at offset 16.
    assert ctypes.sizeof(_lib.Element) == 24
    assert _lib.Element.Z.offset == 16


def _vmap(process=0, precision=0, n=1, element=STANDARD_ROCK, mass=MUON_MASS, ptrs=(0, 0, 0)):
    lib = _lib.load()
    el = _lib.Element(element.A, element.I, element.Z) if element is not None else None
    return lib.noa_dcs_cuda_vmap(process, precision, ptrs[0], ptrs[1], ptrs[2], n,
                                 ctypes.byref(el) if el is not None else None, mass, None)


def test_argument_errors_need_no_gpu(built):
    assert _vmap(process=4) == 1
    assert _vmap(process=-1) == 1
    assert _vmap(precision=7) == 1
    assert _vmap(n=-5) == 1
    assert _vmap(mass=0.0) == 1
    assert _vmap(mass=float("nan")) == 1
    assert _vmap(element=None) == 1
    assert _lib.load().noa_dcs_last_error().decode()


@pytest.mark.parametrize("A,I,Z", [(0.0, 1e-7, 11), (float("nan"), 1e-7, 11), (22.0, -1.0, 11), (22.0, 1e-7, 0),
                                   (float("inf"), 1e-7, 11)])
def test_invalid_elements(built, A, I, Z):
    from noa_gb300.elements import AtomicElement
    assert _vmap(element=AtomicElement(A, I, Z)) == 2


def test_empty_input_is_a_noop(built):
    assert _vmap(n=0) == 0
    lib = _lib.load()
    el = _lib.Element(22.0, 0.1364e-6, 11)
    assert lib.noa_dcs_vmap_host(1, 0, None, None, None, 0, ctypes.byref(el), MUON_MASS) == 0


def test_host_path_rejects_null_and_overlap(built):
    lib = _lib.load()
    el = _lib.Element(22.0, 0.1364e-6, 11)
    assert lib.noa_dcs_vmap_host(0, 0, None, None, None, 4, ctypes.byref(el), MUON_MASS) == 1
    buf = (ctypes.c_double * 8)()
    base = ctypes.addressof(buf)
    assert lib.noa_dcs_vmap_host(0, 0, base + 8, base, base, 4, ctypes.byref(el), MUON_MASS) == 5


def test_python_surface_type_errors():
    import torch
    from noa_gb300 import dcs
    with pytest.raises(RuntimeError):
        dcs.vmap_bremsstrahlung(torch.zeros(3), torch.zeros(3, dtype=torch.float64),
                                torch.zeros(3, dtype=torch.float64))
    with pytest.raises(RuntimeError):   # CPU tensors are not CUDA tensors
        dcs.vmap_bremsstrahlung(*(torch.zeros(3, dtype=torch.float64) for _ in range(3)))


def test_segment_counts_that_overflow_are_rejected_without_a_gpu(built):
    """Counts whose running sum passes INT64_MAX / 8 would wrap the tile
    ranges; the plan and the allocation-free entry point refuse them before
    any CUDA call."""
    lib = _lib.load()
    els = (_lib.Element * 2)(_lib.element_struct(STANDARD_ROCK), _lib.element_struct(STANDARD_ROCK))
    big = (1 << 63) - 1
    for counts in ([big // 8, 1], [big, big]):
        cnt = (ctypes.c_int64 * 2)(*counts)
        plan = ctypes.c_void_p()
        assert lib.noa_dcs_batch_plan_create(ctypes.byref(plan), 0, 0, 2, els, cnt, MUON_MASS) == 1
        assert b"INT64_MAX" in lib.noa_dcs_batch_last_error()
        assert lib.noa_dcs_cuda_vmap_batched_noalloc(0, 0, 2, els, cnt, MUON_MASS, None, None, None, None) == 1
        assert b"INT64_MAX" in lib.noa_dcs_batch_last_error()
