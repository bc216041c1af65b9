"""Error bounds of the FP64 elementary functions in lean64.cuh, measured on
the GPU against the host libm (numpy, correctly rounded or within 1 ulp).
The functions themselves are within ~1.2 ulp of the exact value (log, exp)
and 0.51 ulp (reciprocal), measured against long double in
tests/test_lean64_host.py; the bars here allow numpy's own rounding."""
import numpy as np
import pytest
import torch

from noa_gb300 import _lib

pytestmark = pytest.mark.gpu


def run(fn, x, y=None):
    lib = _lib.load_diag()
    tx = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    ty = torch.from_numpy(np.ascontiguousarray(y)).cuda() if y is not None else tx
    out = torch.empty_like(tx)
    assert lib.noa_dcs_lean64_eval(fn, tx.data_ptr(), ty.data_ptr(), out.data_ptr(), tx.numel(), None) == 0
    torch.cuda.synchronize()
    return out.cpu().numpy()


def ulps(got, exp):
    """Error in units of the last place of the expected value."""
    exp = np.asarray(exp, dtype=np.float64)
    return np.abs(got - exp) / np.spacing(np.abs(exp))


def sample(rng, n, lo, hi):
    return np.exp(rng.uniform(np.log(lo), np.log(hi), n))


def test_log(cuda_device):
    rng = np.random.default_rng(1)
    x = np.concatenate([sample(rng, 400000, 1e-300, 1e300), 1 + rng.uniform(-1e-2, 1e-2, 200000),
                        1 + rng.uniform(-1e-9, 1e-9, 50000), [1.0, 2.0, 0.5, np.sqrt(2.0)]])
    u = ulps(run(0, x), np.log(x))
    assert u.max() <= 2.0, u.max()
    assert u.mean() <= 0.5
    special = np.array([0.0, -1.0, np.inf, np.nan, 5e-324, -0.0])
    got = run(0, special)
    with np.errstate(all="ignore"):
        exp = np.log(special)
    assert np.array_equal(np.isnan(got), np.isnan(exp)) and np.array_equal(got[~np.isnan(exp)],
                                                                             exp[~np.isnan(exp)])


def test_exp(cuda_device):
    rng = np.random.default_rng(2)
    x = np.concatenate([rng.uniform(-699, 699, 400000), rng.uniform(-1e-3, 1e-3, 100000),
                        rng.uniform(-30, 30, 100000), [0.0, 1.0, -1.0]])
    u = ulps(run(1, x), np.exp(x))
    assert u.max() <= 2.0, u.max()
    assert u.mean() <= 0.5
    special = np.array([800.0, -800.0, np.inf, -np.inf, np.nan])
    got = run(1, special)
    with np.errstate(all="ignore"):
        exp = np.exp(special)
    assert np.array_equal(np.isnan(got), np.isnan(exp)) and np.array_equal(got[~np.isnan(exp)],
                                                                             exp[~np.isnan(exp)])


def test_reciprocal_division_sqrt(cuda_device):
    rng = np.random.default_rng(3)
    b = sample(rng, 300000, 1e-300, 1e300) * rng.choice([-1.0, 1.0], 300000)
    assert ulps(run(2, b), 1.0 / b).max() <= 1.0
    a = sample(rng, 300000, 1e-100, 1e100)
    bd = sample(rng, 300000, 1e-150, 1e150) * rng.choice([-1.0, 1.0], 300000)   # a / b stays a normal double
    assert ulps(run(3, a, bd), a / bd).max() <= 2.0
    x = sample(rng, 300000, 1e-300, 1e300)
    assert ulps(run(4, x), np.sqrt(x)).max() <= 2.0
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324])
    with np.errstate(all="ignore"):
        for fn, ref in ((2, 1.0 / special), (4, np.sqrt(special))):
            got = run(fn, special)
            assert np.array_equal(np.isnan(got), np.isnan(ref))
            assert np.array_equal(got[~np.isnan(ref)], ref[~np.isnan(ref)])


def _bits(a):
    return np.asarray(a, dtype=np.float64).view(np.uint64)


def test_integer_pipe_float_conversion_is_the_cast(cuda_device):
    """fpconv::f32 / f64 (integer-pipe conversions used on every hot path)
    give exactly (double)(float)x: round to nearest even, ties, float
    subnormals, overflow to infinity, signed zeros, NaN."""
    rng = np.random.default_rng(7)
    raw = rng.integers(0, 1 << 63, 400_000, dtype=np.uint64).view(np.float64)
    wide = rng.standard_normal(200_000) * 10.0 ** rng.uniform(-50, 45, 200_000)
    f = (rng.standard_normal(50_000) * 10.0 ** rng.uniform(-44, 38, 50_000)).astype(np.float32).astype(np.float64)
    fb = f.view(np.uint64)
    ties = np.concatenate([fb + (1 << 28), fb - (1 << 28), fb + (1 << 28) + 1]).view(np.float64)
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-45, 7e-46, 1.4e-45, 3.4028235e38, 3.4028236e38,
                        -3.5e38, 1.1754943e-38, 1.1754942e-38, 5.877472e-39, 1e-320, 1e300])
    x = np.concatenate([raw, wide, ties, special])
    got = run(5, x)
    with np.errstate(over="ignore", invalid="ignore"):
        exp = x.astype(np.float32).astype(np.float64)
    nan = np.isnan(exp)
    assert np.array_equal(np.isnan(got), nan)
    assert np.array_equal(_bits(got[~nan]), _bits(exp[~nan]))


def test_normal_range_float_conversion(cuda_device):
    """fpconv::f32_normal (the bound checks' conversion): exactly the cast
    (double)(float)x for |x| in [2^-126, 2^128), including ties, carries into
    the exponent and to infinity; NaN for every other input (zeros, float
    subnormals, larger values, infinities, NaN), so that range tests fail."""
    rng = np.random.default_rng(9)
    raw = rng.integers(0, 1 << 63, 400_000, dtype=np.uint64).view(np.float64)
    wide = rng.standard_normal(200_000) * 10.0 ** rng.uniform(-50, 45, 200_000)
    f = (rng.standard_normal(50_000) * 10.0 ** rng.uniform(-37, 38, 50_000)).astype(np.float32).astype(np.float64)
    fb = f.view(np.uint64)
    ties = np.concatenate([fb + (1 << 28), fb - (1 << 28), fb + (1 << 28) + 1]).view(np.float64)
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-45, 1.1754943508222875e-38, 1.1754942e-38,
                        2.0 ** -126, -(2.0 ** -126), 2.0 ** 128, np.nextafter(2.0 ** 128, 0), 3.4028235e38, 1e300])
    x = np.concatenate([raw, wide, ties, special])
    got = run(9, x)
    ax = np.abs(x)
    normal = (ax >= 2.0 ** -126) & (ax < 2.0 ** 128)
    with np.errstate(over="ignore", invalid="ignore"):
        exp = x.astype(np.float32).astype(np.float64)
    assert np.all(np.isnan(got[~normal]))
    assert np.array_equal(_bits(got[normal]), _bits(exp[normal]))


def test_integer_pipe_int_conversion_is_the_cast(cuda_device):
    rng = np.random.default_rng(8)
    i = np.concatenate([rng.integers(-(1 << 31), 1 << 31, 200_000), [0, 1, -1, 2**31 - 1, -2**31, 1023, -1074]])
    x = i.astype(np.float64)
    assert np.array_equal(_bits(run(6, x)), _bits(x))


def float_pair(x):
    """x as the float pair h + l of the float-float split, in extended
    precision (numpy longdouble)."""
    h = x.astype(np.float32)
    l_ = (x - h.astype(np.float64)).astype(np.float32)
    return h.astype(np.longdouble) + l_.astype(np.longdouble)


def test_float_float_exp(cuda_device):
    """ff_exp (Tang's table method on float pairs) to a few 2^-44 of exp of
    its float-pair input, against numpy's extended-precision exp."""
    rng = np.random.default_rng(7)
    x = np.concatenate([rng.uniform(-70, 80, 200000), rng.uniform(-1e-3, 1e-3, 50000), rng.uniform(-25, 0, 200000),
                        [0.0, 1.0, -1.0, np.log(2.0)]])
    got = run(7, x).astype(np.longdouble)
    ref = np.exp(float_pair(x))
    rel = np.abs((got - ref) / ref).astype(np.float64)
    assert rel.max() <= 5e-13, rel.max()


def test_float_float_log(cuda_device):
    """ff_log (float log plus one correction through ff_exp): a few 2^-44
    relative away from 1, ~2^-47 absolute near 1."""
    rng = np.random.default_rng(8)
    x = np.concatenate([sample(rng, 200000, 1e-30, 1e30), 3 + sample(rng, 100000, 1e-6, 1e8),
                        1 + rng.uniform(-1e-3, 1e-3, 100000), [1.0, 2.0, 3.0, 0.5]])
    got = run(8, x).astype(np.longdouble)
    ref = np.log(float_pair(x))
    err = np.abs(got - ref).astype(np.float64)
    big = np.abs(ref) > 0.1
    assert (err[big] / np.abs(ref[big]).astype(np.float64)).max() <= 5e-13
    assert err[~big].max() <= 3e-14


def test_device_equals_host_build(cuda_device, tmp_path):
    """lean_log and lean_exp on the GPU give the bits of the same source
    compiled for the host (tests/lean64_host_check.cu, `values` mode) on
    their fast paths (positive normal x for log, |x| < 700 for exp): the
    functions are integer and float arithmetic with explicit FMAs, so the
    host accuracy study (tests/test_lean64_host.py) describes the device
    code exactly."""
    import os
    import shutil
    import subprocess
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    exe = str(tmp_path / "lean64_host_check")
    subprocess.run([nvcc, "-std=c++17", "-O2", "-Xcompiler", "-ffp-contract=off", "-o", exe,
                    os.path.join(root, "tests", "lean64_host_check.cu")], check=True, capture_output=True)
    rng = np.random.default_rng(17)
    raw = rng.integers(0, 1 << 63, 300_000, dtype=np.uint64).view(np.float64)
    x = np.concatenate([raw[np.isfinite(raw)], sample(rng, 300_000, 1e-300, 1e300), rng.uniform(-745, 745, 300_000),
                        1 + rng.uniform(-1e-3, 1e-3, 100_000), [0.0, -0.0, 1.0, 2.0, np.inf, -np.inf, np.nan]])
    fin, fout = str(tmp_path / "x.bin"), str(tmp_path / "y.bin")
    x.tofile(fin)
    subprocess.run([exe, "values", fin, fout], check=True, timeout=600)
    host = np.fromfile(fout, dtype=np.float64)
    hlog, hexp = host[:x.size], host[x.size:]
    # the fast paths (outside them each build calls its own platform's libm)
    fast = {0: np.isfinite(x) & (x >= 2.0 ** -1022), 1: np.abs(x) < 700}
    for fn, h in ((0, hlog), (1, hexp)):
        d = run(fn, x)
        m = fast[fn]
        same = _bits(d[m]) == _bits(h[m])
        assert m.sum() > 500_000 and same.all(), (fn, int((~same).sum()), x[m][~same][:5])
