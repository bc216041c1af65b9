"""The target workload: 1e8 seeded (K, q) pairs of standard rock for a muon,
the pairs bench.py times (offset 0 of the seeded stream).

* FP64: on a seeded sample of 1e6 of the pairs, the reference's mean metric
  (src/noa/utils/common.hh:228-236) <= 1e-12 against the oracle, every point
  within the conditioning bar of tests/parity.py, identical zero pattern.
* FP32C: against the FP64 output over all 1e8 pairs, max relative error
  <= 1e-6 and identical zero and non-finite patterns.
"""
import numpy as np
import pytest
import torch

import oracle
from noa_gb300 import dcs
from noa_gb300.elements import MUON_MASS, STANDARD_ROCK
from noa_gb300.workload import kinetic_recoil
from tests.parity import PROCESSES, assert_fp64_parity

pytestmark = pytest.mark.gpu

N = 100_000_000
FP32C_TOL = 1e-6


@pytest.fixture(scope="module")
def pairs(cuda_device):
    K, q = kinetic_recoil(N)
    idx = np.sort(np.random.default_rng(31).choice(N, 1_000_000, replace=False))
    tk, tq = torch.from_numpy(K).cuda(), torch.from_numpy(q).cuda()
    yield tk, tq, idx, K[idx], q[idx]
    del tk, tq
    torch.cuda.empty_cache()


@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
def test_fp64_and_fp32c_at_1e8(pairs, process):
    tk, tq, idx, Ks, qs = pairs
    out64 = torch.empty_like(tk)
    dcs.vmap(process, out64, tk, tq, STANDARD_ROCK, MUON_MASS, "fp64")
    out32 = torch.empty_like(tk)
    dcs.vmap(process, out32, tk, tq, STANDARD_ROCK, MUON_MASS, "fp32c")
    torch.cuda.synchronize()

    got = out64[torch.from_numpy(idx).cuda()].cpu().numpy()
    exp = oracle.dcs(process, Ks, qs, STANDARD_ROCK, MUON_MASS)
    s = assert_fp64_parity(got, exp, f"{PROCESSES[process]} 1e8 sample",
                           inputs=(process, Ks, qs, STANDARD_ROCK, MUON_MASS))
    print(PROCESSES[process], "fp64 vs oracle", s)

    assert torch.equal(out32 == 0, out64 == 0), "FP32C zero pattern differs from FP64"
    assert torch.equal(torch.isfinite(out32), torch.isfinite(out64))
    worst = 0.0
    for s in range(0, N, 1 << 24):  # bounded temporaries
        a, b = out32[s:s + (1 << 24)], out64[s:s + (1 << 24)]
        m = (b != 0) & torch.isfinite(b)
        if bool(m.any()):
            worst = max(worst, float(((a[m] - b[m]).abs() / b[m].abs()).max()))
    assert worst <= FP32C_TOL, (PROCESSES[process], worst)
    print(PROCESSES[process], "fp32c max rel vs fp64", worst)
    del out64, out32
