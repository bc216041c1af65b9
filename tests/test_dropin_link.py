"""Link-level proof of the C++ drop-in, on the CPU.

oracle/ref_dropin_caller.cc includes only the reference's own
src/noa/pms/dcs.hh (its noa::pms::dcs::cuda declarations, dcs.hh:1004-1019)
and calls vmap_bremsstrahlung and map_bremsstrahlung.  oracle/build_ref.sh
links it with noa_gb300/libnoa_dcs_torch.so and no header of this repository
on the include path.  An executable links only if every symbol resolves, so a
built caller shows that the library exports the reference's mangled names;
this test also reads those names from both files.  The GPU run of the same
program is in test_gpu_reference.py.
"""
import os
import shutil
import subprocess

import pytest

import oracle
from noa_gb300 import build

STAGED = os.path.join(build.ORACLE_DIR, "_ref", "src", "noa", "pms", "dcs.hh")
SYMBOLS = ("_ZN3noa3pms3dcs4cuda19vmap_bremsstrahlungERKN2at6TensorES6_S6_RKNS0_13AtomicElementERKd",
           "_ZN3noa3pms3dcs4cuda18map_bremsstrahlungERKN2at6TensorES6_RKNS0_13AtomicElementERKd")


def _dynsyms(path):
    out = subprocess.run(["nm", "-D", path], capture_output=True, text=True, check=True).stdout
    table = {}
    for line in out.splitlines():
        f = line.split()
        if len(f) >= 2:
            table[f[-1]] = f[-2]
    return table


@pytest.fixture(scope="module")
def caller(built):
    if shutil.which("nm") is None:
        pytest.skip("nm not available")
    if not os.path.exists(oracle.REF_CALLER):
        build.build_all(ref=False, torch_layer=True)
        if not os.path.exists(STAGED) and not os.environ.get("NOA_CHECKOUT"):
            build.build_ref("all")  # stages the reference headers where a checkout exists
        build.build_ref("caller")
    if not os.path.exists(oracle.REF_CALLER):
        pytest.skip("no noa checkout or staged reference headers: the caller cannot be built")
    return oracle.REF_CALLER


def test_caller_takes_the_reference_symbols_from_the_drop_in(caller):
    theirs = _dynsyms(caller)
    ours = _dynsyms(build.TORCH_LIB)
    for sym in SYMBOLS:
        assert theirs.get(sym) == "U", f"the caller does not import {sym}"
        assert ours.get(sym) == "T", f"libnoa_dcs_torch.so does not define {sym}"


def test_caller_resolves_the_drop_in_library(caller):
    out = subprocess.run(["ldd", caller], capture_output=True, text=True).stdout
    line = next((x for x in out.splitlines() if "libnoa_dcs_torch.so" in x), "")
    assert "=>" in line and "not found" not in line, out
    assert os.path.realpath(line.split("=>")[1].split("(")[0].strip()) == os.path.realpath(build.TORCH_LIB)
