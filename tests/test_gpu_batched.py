"""GPU tests of the batched multi-element engine (noa_dcs_batch_plan_*):
every segment matches the single-element oracle, for FP64 (parity bar) and
FP32C (tolerance), with uneven and empty segments, graph replay, and the
autotuner."""
import ctypes
import json

import numpy as np
import pytest
import torch

import oracle
from noa_gb300 import _lib
from noa_gb300.batched import BatchPlan, batch_inputs
from noa_gb300.elements import BATCH_Z, ELEMENTS, MUON_MASS
from noa_gb300.workload import element_counts
from tests.parity import PROCESSES, assert_fp64_parity, rel_stats

pytestmark = pytest.mark.gpu


def segment_oracle(process, zs, counts, K, q):
    outs, o = [], 0
    for z, c in zip(zs, counts):
        outs.append(oracle.dcs(process, K[o:o + c], q[o:o + c], ELEMENTS[z], MUON_MASS))
        o += c
    return outs


def run_plan(process, zs, counts, precision="fp64", graph=False, tile=None):
    K, q = batch_inputs(zs, counts)
    tk, tq = torch.from_numpy(K).cuda(), torch.from_numpy(q).cuda()
    out = torch.full_like(tk, -7.0)
    with BatchPlan(process, [ELEMENTS[z] for z in zs], counts, precision=precision) as plan:
        if tile:
            plan.set_tile(*tile)
        (plan.execute_graph if graph else plan.execute)(out, tk, tq)
        torch.cuda.synchronize()
    return K, q, out.cpu().numpy()


SMALL_COUNTS = [int(c) for c in element_counts(10, lo=1e2, hi=3e5)]


@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_ten_elements_uneven(cuda_device, process, precision):
    K, q, got = run_plan(process, BATCH_Z, SMALL_COUNTS, precision)
    assert not np.any(got == -7.0)
    o = 0
    for z, c, exp in zip(BATCH_Z, SMALL_COUNTS, segment_oracle(process, BATCH_Z, SMALL_COUNTS, K, q)):
        seg = got[o:o + c]
        Ks, qs = K[o:o + c], q[o:o + c]
        o += c
        if precision == "fp64":
            assert_fp64_parity(seg, exp, f"Z={z}", inputs=(process, Ks, qs, ELEMENTS[z], MUON_MASS))
        else:
            s = rel_stats(seg, exp)
            assert s["zero_agree"] and s["max"] <= 1e-6, (z, s)


@pytest.mark.parametrize("tile", [(128, 1, 1), (128, 8, 2), (256, 2, 3), (256, 8, 1)])
def test_tile_shapes_agree(cuda_device, tile):
    counts = [5000, 0, 12345, 1, 777]
    zs = [1, 6, 11, 26, 82]
    _, _, a = run_plan(1, zs, counts, "fp64", tile=tile)
    _, _, b = run_plan(1, zs, counts, "fp64")
    assert np.array_equal(a, b)


def test_graph_replay_and_recapture(cuda_device):
    zs, counts = [8, 13, 29], [40000, 3000, 90001]
    K, q = batch_inputs(zs, counts)
    tk, tq = torch.from_numpy(K).cuda(), torch.from_numpy(q).cuda()
    with BatchPlan(2, [ELEMENTS[z] for z in zs], counts) as plan:
        ref = plan.execute(torch.empty_like(tk), tk, tq).clone()
        out1 = torch.zeros_like(tk)
        out2 = torch.zeros_like(tk)
        plan.execute_graph(out1, tk, tq)
        plan.execute_graph(out1, tk, tq)   # replay
        plan.execute_graph(out2, tk, tq)   # new buffer -> new capture
        torch.cuda.synchronize()
    assert torch.equal(out1, ref) and torch.equal(out2, ref)


def test_autotune_and_cache(cuda_device, tmp_path):
    zs = list(BATCH_Z)
    K, q = batch_inputs(zs, SMALL_COUNTS)
    tk, tq = torch.from_numpy(K).cuda(), torch.from_numpy(q).cuda()
    cache = tmp_path / "tune.json"
    with BatchPlan(1, [ELEMENTS[z] for z in zs], SMALL_COUNTS, precision="fp32c") as plan:
        tile = plan.autotune(torch.empty_like(tk), tk, tq, sample_per_segment=20000, cache=str(cache))
        assert tile[0] in (128, 256) and 1 <= tile[1] <= 8 and tile[2] >= 1
        assert list(json.loads(cache.read_text()).values()) == [list(tile)]
        out = plan.execute(torch.empty_like(tk), tk, tq)
        torch.cuda.synchronize()
    o = 0
    for z, c, exp in zip(zs, SMALL_COUNTS, segment_oracle(1, zs, SMALL_COUNTS, K, q)):
        s = rel_stats(out.cpu().numpy()[o:o + c], exp)
        o += c
        assert s["zero_agree"] and s["max"] <= 1e-6


def test_plan_argument_errors(cuda_device):
    lib = _lib.load()
    h = ctypes.c_void_p()
    els = (_lib.Element * 17)(*[_lib.Element(22.0, 1e-7, 11)] * 17)
    cnt = (ctypes.c_int64 * 17)(*[10] * 17)
    assert lib.noa_dcs_batch_plan_create(ctypes.byref(h), 0, 0, 17, els, cnt, MUON_MASS) == 1
    assert lib.noa_dcs_batch_plan_create(ctypes.byref(h), 0, 0, 0, els, cnt, MUON_MASS) == 1
    bad = (_lib.Element * 1)(_lib.Element(22.0, 1e-7, 0))
    assert lib.noa_dcs_batch_plan_create(ctypes.byref(h), 0, 0, 1, bad, cnt, MUON_MASS) == 2
    with BatchPlan(0, [ELEMENTS[11]], [100]) as plan:
        d = torch.zeros(100, dtype=torch.float64, device="cuda")
        hst = torch.zeros(100, dtype=torch.float64)
        assert lib.noa_dcs_batch_plan_execute(plan._h, d.data_ptr(), hst.data_ptr(), d.data_ptr(), None) == 4
        assert lib.noa_dcs_batch_plan_set_tile(plan._h, 64, 4, 1) == 1
        assert lib.noa_dcs_batch_plan_set_tolerance(plan._h, ctypes.c_float(0.0)) == 1


def test_all_segments_empty(cuda_device):
    with BatchPlan(0, [ELEMENTS[11], ELEMENTS[1]], [0, 0]) as plan:
        e = torch.zeros(0, dtype=torch.float64, device="cuda")
        plan.execute(e, e, e)
        plan.execute_graph(e, e, e)
