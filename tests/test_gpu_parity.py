"""GPU parity tests of the FP64 kernels, called through the C ABI
(noa_gb300._lib -> libnoa_dcs.so) and checked against the CPU oracle and the
reference's golden vectors."""
import ctypes
import json

import numpy as np
import pytest
import torch

import oracle
from noa_gb300 import _lib, dcs
from noa_gb300.elements import ELEMENTS, MUON_MASS, STANDARD_ROCK, TAU_MASS, AtomicElement
from noa_gb300.workload import kinetic_recoil
from tests.parity import PROCESSES, assert_fp64_parity, rel_stats, same_bits, same_or_both_nan

pytestmark = pytest.mark.gpu


def gpu_dcs(process, K, q, element=STANDARD_ROCK, mass=MUON_MASS, precision="fp64"):
    dev = torch.device("cuda:0")
    tk = torch.as_tensor(np.ascontiguousarray(K), dtype=torch.float64).to(dev)
    tq = torch.as_tensor(np.ascontiguousarray(q), dtype=torch.float64).to(dev)
    out = torch.full_like(tk, -7.0)  # sentinel: every element must be written
    dcs.vmap(process, out, tk, tq, element, mass, precision)
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
@pytest.mark.parametrize("z", [1, 6, 11, 26, 82])
def test_seeded_parity_fp64(cuda_device, process, z):
    K, q = kinetic_recoil(1 << 16, offset=1 << 20)
    el = ELEMENTS[z]
    s = assert_fp64_parity(gpu_dcs(process, K, q, el), oracle.dcs(process, K, q, el, MUON_MASS),
                           f"{PROCESSES[process]} Z={z}", inputs=(process, K, q, el, MUON_MASS))
    print(PROCESSES[process], z, s)


@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
def test_tau_mass_parity(cuda_device, process):
    K, q = kinetic_recoil(1 << 14, offset=3 << 20)
    assert_fp64_parity(gpu_dcs(process, K, q, STANDARD_ROCK, TAU_MASS),
                       oracle.dcs(process, K, q, STANDARD_ROCK, TAU_MASS), PROCESSES[process],
                       inputs=(process, K, q, STANDARD_ROCK, TAU_MASS))


@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
@pytest.mark.parametrize("subset", ["seeded", "notebook", "edge"])
def test_golden_vectors(cuda_device, golden, process, subset):
    meta = json.loads(str(golden["meta"]))
    for ename, (A, I, Z) in meta["elements"].items():
        key = f"{subset}_{ename}_{PROCESSES[process]}"
        if key not in golden:
            continue
        el = AtomicElement(A, I, Z)
        K, q = golden[f"{subset}_K"], golden[f"{subset}_q"]
        got = gpu_dcs(process, K, q, el)
        assert_fp64_parity(got, golden[key], key, inputs=(process, K, q, el, MUON_MASS))


@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
@pytest.mark.parametrize("n", [1, 2, 31, 32, 33, 255, 257, 1023, 1024, 1025, 4097, 70001])
def test_ragged_sizes(cuda_device, process, n):
    K, q = kinetic_recoil(n, offset=999)
    got = gpu_dcs(process, K, q)
    assert not np.any(got == -7.0)
    assert_fp64_parity(got, oracle.dcs(process, K, q, STANDARD_ROCK, MUON_MASS), f"n={n}",
                       inputs=(process, K, q, STANDARD_ROCK, MUON_MASS))


@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
def test_empty(cuda_device, process):
    out = dcs.map(process, torch.zeros(0, dtype=torch.float64, device="cuda"),
                  torch.zeros(0, dtype=torch.float64, device="cuda"))
    assert out.numel() == 0


@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
def test_special_values_propagate_like_the_cpu(cuda_device, process):
    K = np.array([np.nan, 1.0, np.inf, 0.0, 1.0, 10.0, -1.0, 1e6, 1e-3])
    q = np.array([1.0, np.nan, 1.0, 1e-3, 0.0, -1.0, 0.5, np.inf, 1e-3])
    got = gpu_dcs(process, K, q)
    exp = oracle.dcs(process, K, q, STANDARD_ROCK, MUON_MASS)
    assert same_or_both_nan(np.isnan(got), np.isnan(exp))
    assert np.array_equal(np.isfinite(got), np.isfinite(exp))
    fin = np.isfinite(exp)
    s = rel_stats(got[fin], exp[fin])
    assert s["zero_agree"] and s["max"] <= 1e-8


@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
def test_result_may_alias_an_input(cuda_device, process):
    K, q = kinetic_recoil(50000, offset=17)
    tk = torch.from_numpy(K).cuda()
    tq = torch.from_numpy(q).cuda()
    dcs.vmap(process, tk, tk, tq)   # result written over K, as the reference allows
    torch.cuda.synchronize()
    assert_fp64_parity(tk.cpu().numpy(), oracle.dcs(process, K, q, STANDARD_ROCK, MUON_MASS), "alias",
                       inputs=(process, K, q, STANDARD_ROCK, MUON_MASS))


def test_error_paths_with_device_memory(cuda_device):
    lib = _lib.load()
    el = _lib.Element(22.0, 0.1364e-6, 11)
    d = torch.zeros(64, dtype=torch.float64, device="cuda")
    h = torch.zeros(64, dtype=torch.float64)
    p = d.data_ptr()
    # host memory is refused before any launch
    assert lib.noa_dcs_cuda_vmap(0, 0, p, h.data_ptr(), p, 8, ctypes.byref(el), MUON_MASS, None) == 4
    # misaligned pointer
    assert lib.noa_dcs_cuda_vmap(0, 0, p, p + 4, p + 256, 8, ctypes.byref(el), MUON_MASS, None) == 3
    # partial overlap of result and K
    assert lib.noa_dcs_cuda_vmap(0, 0, p + 8, p, p + 256, 8, ctypes.byref(el), MUON_MASS, None) == 5
    assert b"overlap" in lib.noa_dcs_last_error()
    with pytest.raises(RuntimeError):
        dcs.vmap_bremsstrahlung(d[:3], d[:4], d[:4])  # size mismatch
    with pytest.raises(RuntimeError):
        dcs.vmap_bremsstrahlung(d[::2], d[:32], d[:32])  # non-contiguous


@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
@pytest.mark.parametrize("pinned", [False, True])
def test_host_buffer_path(cuda_device, process, pinned):
    n = (1 << 21) * 2 + 12345  # several pipeline chunks plus a tail
    K, q = kinetic_recoil(n, offset=7 << 20)
    tk, tq = torch.from_numpy(K), torch.from_numpy(q)
    out = torch.empty_like(tk)
    if pinned:
        tk, tq, out = tk.pin_memory(), tq.pin_memory(), out.pin_memory()
    dcs.vmap_host(process, out, tk, tq)
    dev = gpu_dcs(process, K, q)
    assert same_bits(out.numpy(), dev)


@pytest.mark.parametrize("layout", ["pageable_result", "offsets_in_pinned"])
def test_host_buffer_path_mixed(cuda_device, layout):
    """Page-locked buffers are worked on in place only when all three are;
    pinned inputs with a pageable result go through the staging pipeline, and
    slices that start inside a pinned allocation are used in place."""
    n = (1 << 21) + 777
    K, q = kinetic_recoil(n + 64, offset=9 << 20)
    tk, tq = torch.from_numpy(K).pin_memory(), torch.from_numpy(q).pin_memory()
    if layout == "pageable_result":
        a, b, out = tk[:n], tq[:n], torch.empty(n, dtype=torch.float64)
        Ks, qs = K[:n], q[:n]
    else:
        buf = torch.empty(n + 64, dtype=torch.float64).pin_memory()
        a, b, out = tk[64:], tq[64:], buf[64:]
        Ks, qs = K[64:], q[64:]
    for process in range(4):
        dcs.vmap_host(process, out, a, b)
        assert same_bits(out.numpy(), gpu_dcs(process, Ks, qs))


@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
def test_runs_on_the_current_stream(cuda_device, process):
    K, q = kinetic_recoil(300000, offset=4242)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        tk = torch.from_numpy(K).cuda(non_blocking=False)
        tq = torch.from_numpy(q).cuda()
        out = dcs.map(process, tk, tq)
    s.synchronize()
    assert same_bits(out.cpu().numpy(), gpu_dcs(process, K, q))


@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
def test_large_size_properties(cuda_device, process):
    """At the 1e7 workload size: deterministic, permutation-equivariant
    (the compaction queue must not mix pairs up), and a random sample of it
    matches the oracle."""
    n = 10_000_000
    K, q = kinetic_recoil(n)
    tk = torch.from_numpy(K).cuda()
    tq = torch.from_numpy(q).cuda()
    a = dcs.map(process, tk, tq)
    b = dcs.map(process, tk, tq)
    perm = torch.randperm(n, generator=torch.Generator().manual_seed(5)).cuda()
    c = dcs.map(process, tk[perm].contiguous(), tq[perm].contiguous())
    torch.cuda.synchronize()
    assert torch.equal(a, b)
    assert torch.equal(a[perm], c)
    idx = np.random.default_rng(11).choice(n, 200_000, replace=False)
    got = a.cpu().numpy()[idx]
    assert_fp64_parity(got, oracle.dcs(process, K[idx], q[idx], STANDARD_ROCK, MUON_MASS), "1e7 sample",
                       inputs=(process, K[idx], q[idx], STANDARD_ROCK, MUON_MASS))
    assert np.all(np.isfinite(a.cpu().numpy()))


@pytest.mark.parametrize("z", [1, 11, 82])
@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_pair_production_bounds(cuda_device, z, precision):
    """Pair production decides q <= 4 me, q >= K + m (1 - 0.75 sqrt(e) Z^1/3)
    and argmin >= 1 in float first, in float-float (K - q, argmin) where float
    cannot, and in IEEE arithmetic within 1e-10 of a bound: pairs at relative
    distances 1e-16..1e-2 on both sides of the two q bounds, and just above
    q = 4 me where argmin -> 1, keep the reference's zero pattern and values."""
    rng = np.random.default_rng(60 + z)
    el = ELEMENTS[z] if z != 11 else STANDARD_ROCK
    me, m = 0.510998910e-03, MUON_MASS
    z13 = float(el.Z) ** (1.0 / 3.0)
    shift = m * (1.0 - 0.75 * np.sqrt(np.e) * z13)
    n = 200_000
    K = 10 ** rng.uniform(-2, 9, n)
    side = rng.choice([-1.0, 1.0], n)
    rel = 10 ** rng.uniform(-16, -2, n)
    q1 = 4 * me * (1 + side * rel)
    q2 = (K + shift) * (1 + side * rel)
    q3 = 4 * me * (1 + 10 ** rng.uniform(-12, 0, n))
    for q in (q1, q2, q3):
        got = gpu_dcs(1, K, q, el, MUON_MASS, precision)
        exp = oracle.dcs(1, K, q, el, MUON_MASS)
        s = rel_stats(got, exp)
        assert s["zero_agree"] and s["nonfinite_agree"], s
        # values relative to the reference's own conditioning: near these
        # edges a 4e-16 change of K and q moves its output by up to ~40%
        nz = exp != 0
        sens = np.zeros_like(exp)
        for d in (4e-16, -4e-16):
            o = oracle.dcs(1, K * (1 + d), q * (1 - d), el, MUON_MASS)
            sens[nz] = np.maximum(sens[nz], np.abs(o[nz] - exp[nz]) / exp[nz])
        err = np.abs(got[nz] - exp[nz]) / exp[nz]
        floor = 1e-12 if precision == "fp64" else 1e-6
        assert np.all(err <= 64 * sens[nz] + floor), float((err - 64 * sens[nz]).max())
