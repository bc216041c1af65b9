"""The reference's own code beside this repository's on the GPU.

* src/noa/pms/dcs.cuh:30-41, the reference's CUDA bremsstrahlung kernel,
  compiled unmodified for sm_103a (oracle/_ref/libnoa_ref_cuda.so): its output
  on the same device buffers is held to the FP64 bar against the oracle, and
  this repository's kernel to the same bar against it.
* oracle/_ref/ref_dropin_caller, a program compiled against the reference's
  declarations only (src/noa/pms/dcs.hh:1004-1019) and linked with
  libnoa_dcs_torch.so: run on cuda:0, its vmap_bremsstrahlung and
  map_bremsstrahlung results equal the C ABI's bit for bit.

Both products come from oracle/build_ref.sh; where no noa checkout or staged
copy of its headers was present at build time they are absent and these
tests skip, saying so.
"""
import os
import subprocess
import tempfile

import numpy as np
import pytest
import torch

import oracle
from noa_gb300 import _lib
from noa_gb300.elements import MUON_MASS, STANDARD_ROCK
from noa_gb300.workload import kinetic_recoil
from tests.parity import assert_fp64_parity, same_bits

pytestmark = pytest.mark.gpu


def ours(K, q):
    lib = _lib.load()
    tk, tq = torch.from_numpy(K).cuda(), torch.from_numpy(q).cuda()
    out = torch.full_like(tk, -7.0)
    _lib.check(lib.noa_dcs_cuda_vmap(0, 0, out.data_ptr(), tk.data_ptr(), tq.data_ptr(), K.size,
                                     _lib.element_struct(STANDARD_ROCK), MUON_MASS,
                                     torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return out.cpu().numpy()


def reference_cuda(K, q):
    tk, tq = torch.from_numpy(K).cuda(), torch.from_numpy(q).cuda()
    out = torch.full_like(tk, -7.0)
    torch.cuda.synchronize()
    oracle.ref_cuda_bremsstrahlung(out.data_ptr(), tk.data_ptr(), tq.data_ptr(), K.size, STANDARD_ROCK, MUON_MASS)
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.fixture(scope="module")
def ref_cuda(cuda_device):
    if not oracle.ref_cuda_available():
        pytest.skip("oracle/_ref/libnoa_ref_cuda.so not built (no noa checkout or staged headers)")
    return oracle.ref_cuda_lib()


@pytest.mark.parametrize("n", [1, 1000, 1 << 20])
def test_reference_cuda_kernel_against_the_oracle_and_ours(ref_cuda, n):
    K, q = kinetic_recoil(n, offset=5 << 22)
    exp = oracle.dcs(0, K, q, STANDARD_ROCK, MUON_MASS)
    theirs = reference_cuda(K, q)
    mine = ours(K, q)
    inputs = (0, K, q, STANDARD_ROCK, MUON_MASS)
    assert_fp64_parity(theirs, exp, "reference CUDA vs oracle", inputs=inputs)
    assert_fp64_parity(mine, exp, "ours vs oracle", inputs=inputs)
    assert_fp64_parity(mine, theirs, "ours vs reference CUDA")


def test_reference_cuda_kernel_on_the_golden_inputs(ref_cuda, golden):
    for subset in ("seeded", "notebook", "edge"):
        K, q = golden[f"{subset}_K"], golden[f"{subset}_q"]
        theirs = reference_cuda(K, q)
        assert_fp64_parity(ours(K, q), theirs, f"{subset}: ours vs reference CUDA")


@pytest.fixture(scope="module")
def caller(cuda_device):
    if not os.path.exists(oracle.REF_CALLER):
        pytest.skip("oracle/_ref/ref_dropin_caller not built (no noa checkout or staged headers)")
    return oracle.REF_CALLER


@pytest.mark.parametrize("n", [0, 1, 4097, 300_000])
def test_program_built_against_the_reference_runs_on_the_drop_in(caller, n):
    K, q = kinetic_recoil(n, offset=11 << 20)
    with tempfile.TemporaryDirectory() as d:
        fin, fout = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
        with open(fin, "wb") as f:
            np.array([n], dtype=np.int64).tofile(f)
            K.tofile(f)
            q.tofile(f)
        r = subprocess.run([caller, fin, fout], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        got = np.fromfile(fout, dtype=np.float64)
    assert got.size == 2 * n
    vmap_res, map_res = got[:n], got[n:]
    mine = ours(K, q)
    assert same_bits(vmap_res, mine)
    assert same_bits(map_res, mine)
    if n:
        assert_fp64_parity(vmap_res, oracle.dcs(0, K, q, STANDARD_ROCK, MUON_MASS), "drop-in caller",
                           inputs=(0, K, q, STANDARD_ROCK, MUON_MASS))
