"""lean64's log, exp and reciprocal, compiled for the host from the device
source (tests/lean64_host_check.cu), against long double libm on the CPU.

The functions are integer and float arithmetic plus one or two double FMAs,
so the host build computes what the GPU computes; the one difference is the
reciprocal's seed, which on the host is deliberately 1 - 3 ulp off the
rounded 1/x (the MUFU approximation's error range).  The GPU build of the
same functions is checked in tests/test_gpu_lean64.py.
"""
import math
import os
import shutil
import subprocess

import pytest

from noa_gb300 import build

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "lean64_host_check.cu")

# max ulp, mean ulp per input set (measured: log <= 1.17 / 0.30, exp <= 1.0 /
# 0.34, rcp <= 0.502 / 0.25 over 2-6e6 inputs)
BARS = {
    "log_random_bits": (1.25, 0.35), "log_bin_edges": (1.25, 0.35), "log_near_one": (0.51, 0.26),
    "log_sqrt2_split": (1.25, 0.35), "exp_wide": (1.05, 0.36), "exp_half_way": (1.05, 0.36),
    "exp_small": (1.05, 0.36), "rcp_random_bits": (0.51, 0.26), "rcp_mantissa_edges": (0.51, 0.26),
}


@pytest.fixture(scope="module")
def report(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path_factory.mktemp("lean64") / "lean64_host_check")
    subprocess.run([nvcc, "-std=c++17", "-O2", "-Xcompiler", "-ffp-contract=off", "-I",
                    os.path.join(build.ROOT, "include"), "-o", exe, SRC], check=True, capture_output=True)
    out = subprocess.run([exe, "400000"], check=True, capture_output=True, text=True, timeout=600).stdout
    sets, special = {}, []
    for line in out.splitlines():
        f = line.split()
        if f[0] == "special":
            special.append((f[1], float.fromhex(f[2]), float.fromhex(f[3]), float.fromhex(f[4])))
        else:
            sets[f[0]] = (int(f[1]), float(f[2]), float(f[3]))
    return sets, special


@pytest.mark.parametrize("name", sorted(BARS))
def test_ulp_error(report, name):
    sets, _ = report
    n, mx, mean = sets[name]
    assert n > 100_000
    bar_max, bar_mean = BARS[name]
    assert mx <= bar_max, (name, mx)
    assert mean <= bar_mean, (name, mean)


def test_special_values_follow_ieee(report):
    _, special = report
    assert len(special) == 36
    for fn, x, got, exp in special:
        if math.isnan(exp):
            assert math.isnan(got), (fn, x, got)
        else:
            assert got == exp and math.copysign(1, got) == math.copysign(1, exp), (fn, x, got, exp)
