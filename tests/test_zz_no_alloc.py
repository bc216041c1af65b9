"""Allocation-free batched entry point, noa_dcs_cuda_vmap_batched_noalloc.

Some callers of this library cannot let it allocate device memory: an
application that has given all of the GPU's memory to its own arena at
start-up, or a particle-transport loop that may not pay for an allocation's
device synchronisation.  This entry point serves them by keeping its only
scratch, the engine's tile counter, in a static device array.  Its results must equal
those of the plan-based batched entry point, on two calls in a row: the
second call runs on the scratch the first one left behind.
"""
import ctypes

import numpy as np
import pytest
import torch

from noa_gb300 import _lib
from noa_gb300.batched import BatchPlan, batch_inputs
from noa_gb300.elements import ELEMENTS, MUON_MASS
from tests.parity import PROCESSES, assert_fp64_parity, rel_stats

pytestmark = pytest.mark.gpu

ZS = [1, 11, 26, 82]
COUNTS = [3000, 0, 20001, 517]


def noalloc(process, precision, tk, tq, zs=ZS, counts=COUNTS):
    lib = _lib.load()
    els = (_lib.Element * len(zs))(*[_lib.element_struct(ELEMENTS[z]) for z in zs])
    cnt = (ctypes.c_int64 * len(counts))(*counts)
    out = torch.full_like(tk, -7.0)
    st = lib.noa_dcs_cuda_vmap_batched_noalloc(process, precision, len(zs), els, cnt, MUON_MASS, out.data_ptr(),
                                               tk.data_ptr(), tq.data_ptr(),
                                               torch.cuda.current_stream().cuda_stream)
    assert st == 0, lib.noa_dcs_batch_last_error()
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_noalloc_matches_plan_on_two_calls(cuda_device, process, precision):
    K, q = batch_inputs(ZS, COUNTS)
    tk, tq = torch.from_numpy(K).cuda(), torch.from_numpy(q).cuda()
    with BatchPlan(process, [ELEMENTS[z] for z in ZS], COUNTS, precision=precision) as plan:
        plan.set_tile(256, 4, 2)
        ref = plan.execute(torch.empty_like(tk), tk, tq).cpu().numpy()
    prec = _lib.PRECISIONS[precision]
    for call in range(2):
        got = noalloc(process, prec, tk, tq)
        assert not np.any(got == -7.0), f"call {call}: pairs left unwritten"
        if precision == "fp64":
            assert_fp64_parity(got, ref, f"call {call}")
        else:
            s = rel_stats(got, ref)
            assert s["zero_agree"] and s["nonfinite_agree"] and s["max"] <= 1e-6, (call, s)


def test_noalloc_rejects_more_segments_than_its_maximum(cuda_device):
    lib = _lib.load()
    zs, counts = [11] * 17, [10] * 17
    tk = torch.zeros(170, dtype=torch.float64, device="cuda")
    els = (_lib.Element * 17)(*[_lib.element_struct(ELEMENTS[z]) for z in zs])
    cnt = (ctypes.c_int64 * 17)(*counts)
    st = lib.noa_dcs_cuda_vmap_batched_noalloc(0, 0, 17, els, cnt, MUON_MASS, tk.data_ptr(), tk.data_ptr(),
                                               tk.data_ptr(), None)
    assert st == 1
    assert b"maximum 16" in lib.noa_dcs_batch_last_error()
