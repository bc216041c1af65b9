"""Host buffers never reach a kernel: every C entry point that takes device
buffers answers NOA_DCS_ERROR_NOT_DEVICE_MEMORY for a host pointer, before
any launch, and the device stays usable."""
import ctypes

import numpy as np
import pytest
import torch

from noa_gb300 import _lib
from noa_gb300.elements import BATCH_Z, ELEMENTS, MUON_MASS

pytestmark = pytest.mark.gpu


def test_diagnostics_reject_host_buffers(cuda_device):
    lib = _lib.load_diag()
    host = np.zeros(64)
    dev = torch.zeros(64, dtype=torch.float64, device="cuda")
    assert lib.noa_dcs_lean64_eval(0, host.ctypes.data, None, dev.data_ptr(), 64, None) == _lib.ERROR_NOT_DEVICE_MEMORY
    assert lib.noa_dcs_lean64_eval(0, dev.data_ptr(), None, host.ctypes.data, 64, None) == _lib.ERROR_NOT_DEVICE_MEMORY
    flops = ctypes.c_double()
    assert lib.noa_dcs_probe_fma(1, host.ctypes.data, 1, 1, ctypes.byref(flops), None) == _lib.ERROR_NOT_DEVICE_MEMORY
    assert lib.noa_dcs_lean64_eval(0, dev.data_ptr(), None, dev.data_ptr(), 64, None) == _lib.SUCCESS
    torch.cuda.synchronize()


def test_surrogate_entry_points_reject_host_buffers(cuda_device):
    lib = _lib.load()
    m = ctypes.c_void_p()
    assert lib.noa_dcs_mlp_create(ctypes.byref(m), 1, 256) == _lib.SUCCESS
    try:
        n = 1000
        hx = np.zeros((n, 4), dtype=np.float32)
        dout = torch.zeros(n, dtype=torch.float32, device="cuda")
        assert lib.noa_dcs_mlp_predict(m, hx.ctypes.data, dout.data_ptr(), n, None) == _lib.ERROR_NOT_DEVICE_MEMORY
        els = (_lib.Element * 1)(_lib.element_struct(ELEMENTS[BATCH_Z[0]]))
        cnt = (ctypes.c_int64 * 1)(n)
        hK = np.ones(n)
        dK = torch.ones(n, dtype=torch.float64, device="cuda")
        dres = torch.zeros(n, dtype=torch.float64, device="cuda")
        trust = torch.zeros(64 * 64, dtype=torch.uint8, device="cuda")
        st = lib.noa_dcs_mlp_infer(m, trust.data_ptr(), 1, els, cnt, MUON_MASS, dres.data_ptr(), hK.ctypes.data,
                                   dK.data_ptr(), ctypes.c_float(1e-6), None, None)
        assert st == _lib.ERROR_NOT_DEVICE_MEMORY
    finally:
        lib.noa_dcs_mlp_destroy(m)
    torch.cuda.synchronize()
