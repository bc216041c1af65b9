"""GPU tests of the DEL / CEL recoil integrals (noa_dcs_cuda_recoil_integral)
against the reference's golden values and the CPU oracle."""
import numpy as np
import pytest
import torch

import oracle
from noa_gb300 import _lib, dcs
from noa_gb300.elements import ELEMENTS, MUON_MASS, STANDARD_ROCK, X_FRACTION
from noa_gb300.workload import kinetic_recoil
from tests.parity import PROCESSES, assert_fp64_parity

pytestmark = pytest.mark.gpu


def gpu_integral(process, moment, K, xlow=X_FRACTION, element=STANDARD_ROCK, min_points=180):
    tk = torch.from_numpy(np.ascontiguousarray(K)).cuda()
    out = torch.full_like(tk, -7.0)
    dcs.recoil_integral(process, moment, out, tk, xlow, element, MUON_MASS, min_points)
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
@pytest.mark.parametrize("moment", [0, 1], ids=["del", "cel"])
def test_integral_golden(cuda_device, golden, process, moment):
    key = f"integral_rock_{PROCESSES[process]}_{['del', 'cel'][moment]}"
    got = gpu_integral(process, moment, golden["integral_K"])
    assert_fp64_parity(got, golden[key], key)


@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
@pytest.mark.parametrize("moment", [0, 1], ids=["del", "cel"])
@pytest.mark.parametrize("z", [1, 26, 82])
def test_integral_oracle(cuda_device, process, moment, z):
    K, _ = kinetic_recoil(3000, offset=777)
    el = ELEMENTS[z]
    got = gpu_integral(process, moment, K, element=el)
    exp = oracle.recoil_integral(process, moment, K, X_FRACTION, el, MUON_MASS, 180)
    assert_fp64_parity(got, exp, f"{PROCESSES[process]} {moment} Z={z}")


@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
@pytest.mark.parametrize("min_points,xlow", [(1, 0.05), (7, 1e-3), (60, 0.5), (600, 1e-4), (1536, 0.05)])
def test_integral_rule_sizes(cuda_device, process, min_points, xlow):
    K, _ = kinetic_recoil(513, offset=4242)
    got = gpu_integral(process, 0, K, xlow=xlow, min_points=min_points)
    exp = oracle.recoil_integral(process, 0, K, xlow, STANDARD_ROCK, MUON_MASS, min_points)
    assert_fp64_parity(got, exp, f"min_points={min_points} xlow={xlow}")


@pytest.mark.parametrize("n", [1, 7, 8, 9, 1001])
def test_integral_ragged(cuda_device, n):
    K, _ = kinetic_recoil(n, offset=99)
    got = gpu_integral(1, 1, K)
    assert not np.any(got == -7.0)
    assert_fp64_parity(got, oracle.recoil_integral(1, 1, K, X_FRACTION, STANDARD_ROCK, MUON_MASS, 180), "ragged")


def test_integral_argument_errors(cuda_device):
    lib = _lib.load()
    d = torch.zeros(8, dtype=torch.float64, device="cuda")
    el = _lib.element_struct(STANDARD_ROCK)
    call = lambda moment=0, xlow=0.05, mp=180: lib.noa_dcs_cuda_recoil_integral(  # noqa: E731
        0, moment, d.data_ptr(), d.data_ptr(), 8, xlow, el, MUON_MASS, mp, None)
    assert call(moment=2) == 1
    assert call(xlow=0.0) == 1
    assert call(xlow=1.5) == 1
    assert call(mp=0) == 1
    assert call(mp=5000) == 1
