#!/usr/bin/env python3
"""Benchmark of the GB300 muon DCS path (one JSON line on stdout, rank 0).

Workload (one "step"): the four DCS processes of NOA's PMS module --
bremsstrahlung, pair production, photonuclear, ionisation -- evaluated in
plain FP64 over 1e8 seeded (K, q) pairs of standard rock for a muon, i.e.
4e8 DCS evaluations.  This is the reference's benchmark of
benchmark/measure-dcs-calc.cc (vectorised dcs::vmap per process) at the
mixed-precision target size of 1e8 pairs; the pairs follow
K ~ log-uniform[1e-3, 1e6] GeV, nu ~ log-uniform[1e-7, 1], q = nu K
(noa_gb300.workload, seed 987654).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`value` is DCS evaluations per second with inputs resident in HBM (CUDA
events on the launching stream; K and q are 1.6 GB, far above the 129 MB L2,
so no flush is needed between steps).  `e2e` is the same metric through the C
ABI's host-buffer entry point (noa_dcs_vmap_host) from pinned host memory,
host-device traffic included: the kernels read K and q and write the results
in the page-locked host buffers over NVLink-C2C.  Beside it, on the same
pairs: the FP32-compensated form, the reference's own CUDA bremsstrahlung
kernel (src/noa/pms/dcs.cuh, compiled unmodified for sm_103a by
oracle/build_ref.sh), the batched multi-element engine, the learned
surrogate, and the per-K integrals.  `--impl reference` times the reference's
CPU implementation on the host cores: its own dcs::pvmap (src/noa/pms/dcs.hh,
OpenMP over all cores) where oracle/build_ref.sh compiled it, else the CPU
oracle (an operation-for-operation restatement, bit-exact with it).  The
line ends with a compact `summary` of all of these.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DCS evals/sec per process on 1 GB300 (plain FP64 vs FP32-comp vs MLP) at stated rel. error"
PROCESSES = ("bremsstrahlung", "pair_production", "photonuclear", "ionisation")
N_PAIRS = 100_000_000
# Algorithmic work per evaluation on this workload, in flop-equivalents
# (+ - * / sqrt compare = 1, log exp pow log10 = 20), counted by running the
# reference's operation sequence on an op-counting scalar over 1e6 pairs of
# the seeded law (tests/test_bench_contract.py re-derives them).
FLOP_EQ_PER_EVAL = {"bremsstrahlung": 156.27, "pair_production": 1192.49,
                    "photonuclear": 949.69, "ionisation": 57.98}
BYTES_PER_EVAL = 24  # K and q read, result written, float64


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=N_PAIRS)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-reference-cuda", action="store_true")
    ap.add_argument("--no-integrals", action="store_true")
    ap.add_argument("--no-surrogate", action="store_true")
    ap.add_argument("--surrogate-queries", type=int, default=100_000_000)
    return ap.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def shard_offset(rank, n):
    """First workload element of a rank's shard: every rank evaluates its own
    n pairs of the seeded stream (weak scaling, no data exchange)."""
    return rank * n


def reduce_max(value, world, device=None):
    """Max of a float over ranks (the slowest rank's time); identity for one rank."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as tdist
    t = torch.tensor([value], dtype=torch.float64, device=device)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------- CPU side
def cpu_dcs_fn():
    """The CPU implementation timed as the baseline: the reference's own
    dcs::pvmap / dcs::vmap (oracle/_ref/libnoa_ref_dcs_bench.so, compiled from
    src/noa/pms/dcs.hh by oracle/build_ref.sh with the reference benchmark's
    flags: -O3, OpenMP) where it was built on this host, else the oracle port.  Returns (fn, kind) with
    fn(process, K, q, threads) -> out; threads 0 = every host thread
    (dcs::pvmap), 1 = the serial loop (dcs::vmap)."""
    import oracle
    from noa_gb300.elements import MUON_MASS, STANDARD_ROCK
    if oracle.ref_available("bench"):
        try:
            oracle.ref_lib("bench")

            def fn(p, K, q, threads):
                return oracle.ref_dcs(p, K, q, STANDARD_ROCK, MUON_MASS, parallel=threads != 1, build="bench")
            return fn, "reference"
        except OSError:
            pass

    def port(p, K, q, threads):
        return oracle.dcs(p, K, q, STANDARD_ROCK, MUON_MASS, threads=threads)
    return port, "port"


def cpu_reference_rate(n_sample, reps=5, offset=0, threads=0):
    """Evaluations/s of the CPU baseline (cpu_dcs_fn) on the first n_sample
    pairs of the workload, all four processes, median of reps runs after one
    warm-up; threads 0 = every host thread (dcs::pvmap), 1 = the serial loop
    (dcs::vmap)."""
    import oracle
    from noa_gb300.workload import kinetic_recoil
    fn, kind = cpu_dcs_fn()
    K, q = kinetic_recoil(n_sample, offset=offset)
    for p in range(4):
        fn(p, K, q, threads)
    per = {}
    total_t = []
    for _ in range(reps):
        t_all = 0.0
        for p, name in enumerate(PROCESSES):
            t0 = time.perf_counter()
            fn(p, K, q, threads)
            dt = time.perf_counter() - t0
            per.setdefault(name, []).append(dt)
            t_all += dt
        total_t.append(t_all)
    t = statistics.median(total_t)
    return {
        "value": 4 * n_sample / t,
        "seconds_per_sample": t,
        "per_process": {k: n_sample / statistics.median(v) for k, v in per.items()},
        "cores": oracle.lib().oracle_max_threads() if threads == 0 else threads,
        "kind": kind,
    }


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    n_sample = min(args.n, 2_000_000)
    import oracle
    from noa_gb300.workload import kinetic_recoil
    fn, kind = cpu_dcs_fn()
    K, q = kinetic_recoil(n_sample)
    for _ in range(args.warmup):
        for p in range(4):
            fn(p, K, q, 0)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        for p in range(4):
            fn(p, K, q, 0)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = 4 * n_sample * args.steps / total
    cores = oracle.lib().oracle_max_threads()
    what = ("the reference's own dcs::pvmap (src/noa/pms/dcs.hh compiled on this host with its benchmark's "
            "flags, -O3 -fopenmp)"
            if kind == "reference" else "the CPU oracle port of dcs::pvmap (OpenMP)")
    sample = (f"{what}: first {n_sample} pairs of the {args.n:.0e}-pair workload per step, all four processes "
              f"(the pairs are i.i.d., so the rate is the workload's)")
    line = {
        "metric": METRIC, "value": value, "unit": "evals/s", "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded log-uniform K in [1e-3,1e6] GeV, nu in [1e-7,1], q = nu K",
        "config": config_dict(args.n, world),
        "cpu_baseline": {"value": value, "unit": "evals/s", "cores": cores, "kind": kind, "sample": sample},
        "e2e": {"value": value, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def config_dict(n, world):
    return {"workload": f"plain FP64 DCS, 4 processes x {n:.0e} (K,q) pairs, standard rock, muon",
            "n_pairs_per_gpu": n, "processes": list(PROCESSES),
            "element": {"A": 22.0, "I": 0.1364e-6, "Z": 11}, "mass": 0.10565839,
            "parallelism": f"replicas x{world} (independent shards)" if world > 1 else "single GPU",
            "l2": f"inputs {16 * n / 1e9:.3g} GB vs 129 MB L2: "
                  + ("no flush between steps" if 16 * n > 129e6 else "smaller than L2")}


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for name, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------- GPU side
def measure_fp64_peak(torch, stream):
    """FP64 FMA-chain throughput (TFLOP/s) of this GPU: the roofline
    denominator (probe of the instrument library libnoa_dcs_diag.so)."""
    import ctypes
    from noa_gb300 import _lib
    lib = _lib.load_diag()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    blocks = sms * 8
    out = torch.empty(blocks * 256, dtype=torch.float64, device="cuda")
    flops = ctypes.c_double()
    best = 0.0
    for it in (64, 2048, 2048, 2048):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        rc = lib.noa_dcs_probe_fma(1, out.data_ptr(), blocks, it, ctypes.byref(flops), stream.cuda_stream)
        e.record(stream)
        e.synchronize()
        if rc == 0 and it > 64:
            best = max(best, flops.value / (s.elapsed_time(e) * 1e-3) / 1e12)
    return best


def rel_error_stats(torch, got, ref):
    """max / median relative error of got against ref over ref != 0, and
    whether the zero patterns agree."""
    nz = ref != 0
    rel = ((got[nz] - ref[nz]).abs() / ref[nz].abs()).float()
    return {"max_rel": float(rel.max()) if rel.numel() else 0.0,
            "median_rel": float(rel.median()) if rel.numel() else 0.0,
            "mean_rel": float(rel.mean()) if rel.numel() else 0.0,
            "zero_pattern_equal": bool(torch.equal(got == 0, ref == 0))}


def time_fp32c(lib, torch, tk, tq, ref_outs, n, el, mass, stream, args, fp64_s):
    """FP32-compensated form (NOA_DCS_FP32C, tolerance 1e-6) on the same
    pairs: evals/s per process, speed-up over the FP64 kernel, and its error
    against the FP64 kernel's output."""
    from noa_gb300 import _lib
    out = torch.empty_like(tk)
    res = {}
    for p, name in enumerate(PROCESSES):
        def launch():
            _lib.check(lib.noa_dcs_cuda_vmap(p, 1, out.data_ptr(), tk.data_ptr(), tq.data_ptr(), n, el, mass,
                                             stream.cuda_stream))
        for _ in range(args.warmup):
            launch()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        s.record(stream)
        for _ in range(args.steps):
            launch()
        e.record(stream)
        torch.cuda.synchronize()
        t = s.elapsed_time(e) * 1e-3
        res[name] = {"evals_per_s": n * args.steps / t, "ms_per_launch": 1e3 * t / args.steps,
                     "speedup_vs_fp64": fp64_s[name] / t, "tolerance": 1e-6,
                     **rel_error_stats(torch, out, ref_outs[p])}
    total = sum(v["ms_per_launch"] for v in res.values())
    res["all_processes"] = {"evals_per_s": 4 * n / (total * 1e-3),
                            "speedup_vs_fp64": sum(fp64_s.values()) / args.steps / (total * 1e-3)}
    return res


def time_reference_cuda(torch, tk, tq, ours, n, args, sample_idx):
    """The reference's own CUDA kernel, dcs::cuda::vmap_bremsstrahlung
    (src/noa/pms/dcs.cuh:30-41: one thread per pair, legacy default stream),
    compiled unmodified for sm_103a by oracle/build_ref.sh, timed with CUDA
    events on the default stream over the same device-resident pairs as the
    headline; its output is compared with this repository's bremsstrahlung
    over all pairs and with the oracle on the parity sample."""
    import oracle
    from noa_gb300.elements import MUON_MASS, STANDARD_ROCK
    if not oracle.ref_cuda_available():
        return {"available": False,
                "why": "oracle/_ref/libnoa_ref_cuda.so not built (no noa checkout or staged headers at build time)"}
    out = torch.empty_like(tk)
    stream = torch.cuda.default_stream()

    def launch():
        oracle.ref_cuda_bremsstrahlung(out.data_ptr(), tk.data_ptr(), tq.data_ptr(), n, STANDARD_ROCK, MUON_MASS)

    torch.cuda.synchronize()
    for _ in range(max(1, args.warmup)):
        launch()
    steps = max(1, min(args.steps, 5))
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    s.record(stream)
    for _ in range(steps):
        launch()
    e.record(stream)
    torch.cuda.synchronize()
    ms = s.elapsed_time(e) / steps
    res = {"available": True, "ms_per_launch": ms, "evals_per_s": n / (ms * 1e-3),
           "vs_ours": rel_error_stats(torch, out, ours)}
    ref = oracle.dcs(0, *sample_idx[1:], STANDARD_ROCK, MUON_MASS)
    got = out[torch.from_numpy(sample_idx[0]).to(out.device)].cpu().numpy()
    nz = ref != 0
    rel = np.abs(got[nz] - ref[nz]) / np.abs(ref[nz])
    res["vs_oracle_sample"] = {"mean_rel": float(rel.mean()), "max_rel": float(rel.max())}
    del out
    return res


def conditioning_ratio(p, K, q, got, ref, element, mass, delta=4e-16):
    """Largest ratio of a point's relative error to 64 x the reference's own
    response to +-delta relative changes of K and q, plus 1e-12 (the per-point
    parity bar of the tests); <= 1 means every point is within it."""
    import oracle
    ok = np.isfinite(ref) & (ref != 0)
    sens = np.zeros_like(ref)
    for dk in (delta, -delta):
        for dq in (delta, -delta):
            o = oracle.dcs(p, K * (1 + dk), q * (1 + dq), element, mass)
            with np.errstate(invalid="ignore", divide="ignore", over="ignore"):
                r = np.abs(o - ref) / np.abs(ref)
            sens = np.maximum(sens, np.where(ok & np.isfinite(r), r, np.where(ok, np.inf, 0.0)))
    err = np.abs(got[ok] - ref[ok]) / np.abs(ref[ok])
    return float(np.max(err / (64 * sens[ok] + 1e-12))) if ok.any() else 0.0


def time_batched(torch, args):
    """Batched multi-element form: the 10 elements Z in {1,6,8,11,13,14,20,26,
    29,82} with seeded uneven counts (log-uniform in [1e4, 3e7]) in one
    persistent launch per process, tile shape from the autotuner, replayed as
    a CUDA graph; FP64 and FP32C."""
    from noa_gb300.batched import BatchPlan, batch_inputs
    from noa_gb300.elements import BATCH_Z, ELEMENTS, MUON_MASS
    from noa_gb300.workload import element_counts
    counts = [int(c) for c in element_counts()]
    K, q = batch_inputs(BATCH_Z, counts)
    tk, tq = torch.from_numpy(K).cuda(), torch.from_numpy(q).cuda()
    out = torch.empty_like(tk)
    n = tk.numel()
    res = {"elements_Z": list(BATCH_Z), "counts": counts, "total_pairs": n}
    stream = torch.cuda.current_stream()
    for precision in ("fp64", "fp32c"):
        per = {}
        for p, name in enumerate(PROCESSES):
            with BatchPlan(p, [ELEMENTS[z] for z in BATCH_Z], counts, MUON_MASS, precision) as plan:
                tile = plan.autotune(out, tk, tq, sample_per_segment=1 << 17, cache=None)
                for _ in range(max(1, args.warmup)):
                    plan.execute_graph(out, tk, tq)
                s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                steps = max(1, min(args.steps, 5))
                torch.cuda.synchronize()
                s.record(stream)
                for _ in range(steps):
                    plan.execute_graph(out, tk, tq)
                e.record(stream)
                torch.cuda.synchronize()
                t = s.elapsed_time(e) * 1e-3 / steps
                per[name] = {"evals_per_s": n / t, "ms_per_launch": 1e3 * t,
                             "tile": {"threads": tile[0], "items": tile[1], "ctas_per_sm": tile[2]}}
        total_ms = sum(v["ms_per_launch"] for v in per.values())
        per["all_processes"] = {"evals_per_s": 4 * n / (total_ms * 1e-3)}
        res[precision] = per
    return res


def time_integrals(torch, args, with_cpu):
    """DEL / CEL recoil integrals (dcs::vmap_integral(dcs::recoil_integral(...)),
    xlow = 0.05, 180 nodes per K as in the reference's benchmark) over 1e5
    seeded kinetic energies, FP64, per process and moment; the CPU oracle is
    timed on the first 2000 energies with every host thread."""
    from noa_gb300 import dcs
    from noa_gb300.elements import MUON_MASS, STANDARD_ROCK, X_FRACTION
    from noa_gb300.workload import kinetic_recoil
    nk = 100_000
    K, _ = kinetic_recoil(nk, offset=1 << 30)
    tk = torch.from_numpy(K).cuda()
    out = torch.empty_like(tk)
    stream = torch.cuda.current_stream()
    res = {"n_kinetic": nk, "nodes_per_K": 180, "xlow": X_FRACTION}
    for p, name in enumerate(PROCESSES):
        for moment, mname in ((0, "del"), (1, "cel")):
            for _ in range(max(1, args.warmup)):
                dcs.recoil_integral(p, moment, out, tk)
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            steps = max(1, min(args.steps, 5))
            torch.cuda.synchronize()
            s.record(stream)
            for _ in range(steps):
                dcs.recoil_integral(p, moment, out, tk)
            e.record(stream)
            torch.cuda.synchronize()
            t = s.elapsed_time(e) * 1e-3 / steps
            entry = {"K_per_s": nk / t, "ms": 1e3 * t}
            if with_cpu:
                import oracle
                ns = 2000
                t0 = time.perf_counter()
                oracle.recoil_integral(p, moment, K[:ns], X_FRACTION, STANDARD_ROCK, MUON_MASS, 180, threads=0)
                tc = time.perf_counter() - t0
                entry["cpu_port_K_per_s"] = ns / tc
                entry["speedup_vs_cpu"] = entry["K_per_s"] / entry["cpu_port_K_per_s"]
            res[f"{name}_{mname}"] = entry
    return res


def time_transport(torch, args, with_cpu):
    """Per-K transport functions over 1e5 seeded kinetic energies, FP64:
    soft_scattering (dcs.hh:941-952: 102 photonuclear DCS nodes per K) and the
    elastic chain coulomb_data -> coulomb_transport(mu = 1) -> hard_scattering
    (dcs.hh:499-872) for standard rock; the CPU oracle is timed on the first
    5000 energies (soft scattering, every host thread) or all of them
    (elastic chain, one thread: the reference's loops are serial)."""
    import oracle
    from noa_gb300 import dcs
    from noa_gb300.elements import MUON_MASS, STANDARD_ROCK
    from noa_gb300.workload import kinetic_recoil
    nk = 100_000
    K, _ = kinetic_recoil(nk, offset=1 << 31)
    tk = torch.from_numpy(K).cuda()
    out = torch.empty_like(tk)
    f64 = dict(dtype=torch.float64, device="cuda")
    fCM, screen, fspin, il = (torch.empty(nk, 2, **f64), torch.empty(nk, 9, **f64), torch.empty(nk, **f64),
                              torch.empty(nk, **f64))
    G, mu0, lb_h = torch.empty(nk, 2, **f64), torch.empty(nk, **f64), torch.empty(nk, **f64)
    one = torch.tensor(1.0, **f64)

    def soft():
        dcs.soft_scattering(out, tk)

    def chain():
        dcs.coulomb_data(fCM, screen, fspin, il, tk)
        dcs.coulomb_transport(G, screen, fspin, one)
        dcs.hard_scattering(mu0, lb_h, G.view(1, nk, 2), fCM.view(1, nk, 2), screen.view(1, nk, 9),
                            il.view(1, nk), fspin.view(1, nk))

    stream = torch.cuda.current_stream()
    res = {"n_kinetic": nk}
    for name, fn in (("soft_scattering", soft), ("coulomb_chain", chain)):
        for _ in range(max(1, args.warmup)):
            fn()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        steps = max(1, min(args.steps, 5))
        torch.cuda.synchronize()
        s.record(stream)
        for _ in range(steps):
            fn()
        e.record(stream)
        torch.cuda.synchronize()
        t = s.elapsed_time(e) * 1e-3 / steps
        res[name] = {"K_per_s": nk / t, "ms": 1e3 * t}
    if with_cpu:
        ns = 5000
        t0 = time.perf_counter()
        oracle.soft_scattering(K[:ns], STANDARD_ROCK, MUON_MASS, threads=0)
        res["soft_scattering"]["cpu_port_K_per_s"] = ns / (time.perf_counter() - t0)
        t0 = time.perf_counter()
        d = oracle.coulomb_data(K, STANDARD_ROCK, MUON_MASS)
        Gc = oracle.coulomb_transport(d[1], d[2], 1.0)
        oracle.hard_scattering(Gc, d[0], d[1], d[3], d[2])
        res["coulomb_chain"]["cpu_port_K_per_s"] = nk / (time.perf_counter() - t0)
        for v in (res["soft_scattering"], res["coulomb_chain"]):
            v["speedup_vs_cpu"] = v["K_per_s"] / v["cpu_port_K_per_s"]
    return res


def time_surrogate(torch, args):
    """Learned surrogate (pair production, photonuclear): trained here on the
    GPU (plain-kernel data, tensor-core forward / backward, Adam; moderate
    recipe), then evaluated on `surrogate_queries` seeded pairs over the 10
    elements: the network answers the pairs of trusted cells (held-out error
    <= 3.5e-4), the FP32C kernel the rest.  Compared with the plain FP64 kernel
    and the FP32C kernel (batched engine, one launch) on the same pairs; error
    against the plain FP64 output."""
    from noa_gb300.batched import BatchPlan, batch_inputs
    from noa_gb300.elements import BATCH_Z, ELEMENTS, MUON_MASS
    from noa_gb300.surrogate import train_recipe
    nq = args.surrogate_queries
    counts = [nq // len(BATCH_Z)] * len(BATCH_Z)
    counts[-1] += nq - sum(counts)
    K, q = batch_inputs(BATCH_Z, counts, seed=777)
    tk, tq = torch.from_numpy(K).cuda(), torch.from_numpy(q).cuda()
    del K, q
    stream = torch.cuda.current_stream()
    steps = max(1, min(args.steps, 3))
    res = {"queries": nq, "elements_Z": list(BATCH_Z), "error_bound": 1e-3}

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        for _ in range(steps):
            fn()
        e.record(stream)
        torch.cuda.synchronize()
        return s.elapsed_time(e) * 1e-3 / steps

    for p, name in ((1, "pair_production"), (2, "photonuclear")):
        # trained on 2e7 plain-kernel samples over the 10 elements
        sur = train_recipe(p, n_valid=20_000_000, steps1=30_000, steps2=90_000, batch=8192, heldout=2_000_000)
        ref = torch.empty_like(tk)
        out = torch.empty_like(tk)
        entry = {"training": sur.info}
        with BatchPlan(p, [ELEMENTS[z] for z in BATCH_Z], counts, MUON_MASS, "fp64") as plan:
            plan.set_tile(256, 8, 2)
            entry["fp64_s"] = timed(lambda: plan.execute_graph(ref, tk, tq))
        with BatchPlan(p, [ELEMENTS[z] for z in BATCH_Z], counts, MUON_MASS, "fp32c") as plan:
            plan.set_tile(256, 8, 2)
            entry["fp32c_s"] = timed(lambda: plan.execute_graph(out, tk, tq))
        stats = {}

        def run():
            _, st = sur.infer(tk, tq, counts, out=out)
            stats.update(st)
        entry["surrogate_s"] = timed(run)
        # the same pipeline with every cell untrusted: what the network adds
        none = np.zeros_like(sur.trust)
        entry["no_network_s"] = timed(lambda: sur.infer(tk, tq, counts, trust=none, out=out))
        sur.infer(tk, tq, counts, out=out)
        nz = ref != 0
        rel = ((out[nz] - ref[nz]).abs() / ref[nz]).float()
        entry.update({
            "evals_per_s": {"fp64": nq / entry["fp64_s"], "fp32c": nq / entry["fp32c_s"],
                            "surrogate": nq / entry["surrogate_s"]},
            "speedup_vs_fp64": entry["fp64_s"] / entry["surrogate_s"],
            "speedup_vs_fp32c": entry["fp32c_s"] / entry["surrogate_s"],
            "speedup_vs_no_network": entry["no_network_s"] / entry["surrogate_s"],
            "network_share_of_open": stats["network"] / max(1, int(nz.sum())),
            "status": stats["status"],
            "max_rel": float(rel.max()), "median_rel": float(rel.median()),
            "frac_above_1e-3": float((rel > 1e-3).float().mean()),
            "zero_pattern_equal": bool(torch.equal(out == 0, ref == 0)),
        })
        res[name] = entry
        sur.close()
        del ref, out
    return res


def load_traffic():
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def hw_view(process):
    """The hardware view of the roofline for one FP64 kernel: ncu's pipe
    utilisations of a 1e7-pair launch (profiles/traffic.json), the FP64 pipe
    being the bound."""
    pipes = load_traffic().get("pipes_fp64_1e7", {}).get(process)
    if not pipes:
        return None
    return {"bound": "fp64 pipe", "frac": pipes["fp64_pipe"], "pipes": pipes,
            "source": "ncu --set full of one 1e7-pair launch (profiles/dcs_fp64_1e8.md)"}


def run_ours(args):
    import numpy as np
    import torch
    import torch.distributed as tdist
    from noa_gb300 import _lib
    from noa_gb300.elements import MUON_MASS, STANDARD_ROCK
    from noa_gb300.workload import kinetic_recoil

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        tdist.init_process_group("nccl", device_id=torch.device("cuda", local))
    lib = _lib.load()
    n = args.n
    K, q = kinetic_recoil(n, offset=shard_offset(rank, n))  # each rank its own shard: weak scaling
    dev = torch.device("cuda", local)
    tk = torch.from_numpy(K).to(dev)
    tq = torch.from_numpy(q).to(dev)
    outs = [torch.empty_like(tk) for _ in PROCESSES]
    el = _lib.element_struct(STANDARD_ROCK)
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream

    def step(ev=None):
        for p in range(4):
            if ev is not None:
                ev[p][0].record(stream)
            _lib.check(lib.noa_dcs_cuda_vmap(p, 0, outs[p].data_ptr(), tk.data_ptr(), tq.data_ptr(), n, el,
                                             MUON_MASS, sptr))
            if ev is not None:
                ev[p][1].record(stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    evs = [[[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(4)]
           for _ in range(args.steps)]
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if world > 1:
        tdist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        start.record(stream)
        for s in range(args.steps):
            step(evs[s])
        end.record(stream)
        torch.cuda.synchronize()
    if world > 1:
        tdist.barrier()
    elapsed = start.elapsed_time(end) * 1e-3
    per_proc_s = {name: sum(evs[s][p][0].elapsed_time(evs[s][p][1]) for s in range(args.steps)) * 1e-3
                  for p, name in enumerate(PROCESSES)}
    elapsed = reduce_max(elapsed, world, dev)
    value = world * 4 * n * args.steps / elapsed

    # parity of the timed outputs: a seeded sample of 1e5 pairs against the
    # oracle (the reference's algorithm, bit-exact with it on the CPU): the
    # reference's mean metric, the max, the zero pattern, and the per-point
    # conditioning bar of the tests (cond_ratio <= 1)
    parity = None
    sample = None
    if rank == 0:
        import oracle
        idx = np.sort(np.random.default_rng(2024).choice(n, min(n, 100_000), replace=False))
        sample = (idx, K[idx], q[idx])
        ti = torch.from_numpy(idx).to(dev)
        parity = {"sample": f"{len(idx)} seeded indices of the timed step's pairs"}
        for p, name in enumerate(PROCESSES):
            got = outs[p][ti].cpu().numpy()
            ref = oracle.dcs(p, K[idx], q[idx], STANDARD_ROCK, MUON_MASS)
            nz = ref != 0
            rel = np.abs(got[nz] - ref[nz]) / np.abs(ref[nz]) if nz.any() else np.zeros(1)
            parity[name] = {"mean_rel": float(rel.mean()), "max_rel": float(rel.max()),
                            "zero_pattern_equal": bool(np.array_equal(got == 0, ref == 0)),
                            "cond_ratio": conditioning_ratio(p, K[idx], q[idx], got, ref, STANDARD_ROCK,
                                                             MUON_MASS)}

    # e2e: host buffers in pinned memory, through noa_dcs_vmap_host, host-device traffic timed.
    e2e = None
    if not args.no_e2e:
        hk = torch.from_numpy(K).pin_memory()
        hq = torch.from_numpy(q).pin_memory()
        hout = [torch.empty(n, dtype=torch.float64).pin_memory() for _ in PROCESSES]

        def host_step():
            for p in range(4):
                _lib.check(lib.noa_dcs_vmap_host(p, 0, hout[p].data_ptr(), hk.data_ptr(), hq.data_ptr(), n, el,
                                                 MUON_MASS))
        host_step()
        e2e_steps = max(1, min(args.steps, 5))
        if world > 1:
            tdist.barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            host_step()
        t_e2e = time.perf_counter() - t0
        t_e2e = reduce_max(t_e2e, world, dev)
        e2e = {"value": world * 4 * n * e2e_steps / t_e2e, "unit": "evals/s",
               "h2d_bytes_per_step": 4 * 2 * 8 * n, "d2h_bytes_per_step": 4 * 8 * n, "steps": e2e_steps,
               "path": "noa_dcs_vmap_host (pinned host buffers read and written in place by the kernels over NVLink-C2C)"}
        # correctness of the timed e2e results against the device path
        for p in range(4):
            if not torch.equal(hout[p], outs[p].cpu()):
                raise RuntimeError(f"e2e result differs from device result for {PROCESSES[p]}")
        del hk, hq, hout

    variants = {"fp64": {name: {"evals_per_s": n * args.steps / t} for name, t in per_proc_s.items()}}
    variants["fp32c"] = time_fp32c(lib, torch, tk, tq, outs, n, el, MUON_MASS, stream, args, per_proc_s)

    if rank != 0:
        if world > 1:
            tdist.destroy_process_group()
        return

    ref_cuda = None
    if not args.no_reference_cuda:
        ref_cuda = time_reference_cuda(torch, tk, tq, outs[0], n, args, sample)
        if ref_cuda.get("available"):
            ref_cuda["ours_ms_per_launch"] = 1e3 * per_proc_s["bremsstrahlung"] / args.steps
            ref_cuda["speedup_of_ours"] = ref_cuda["ms_per_launch"] / ref_cuda["ours_ms_per_launch"]
    del tk, tq, outs
    torch.cuda.empty_cache()

    peak = measure_fp64_peak(torch, stream)
    dom = max(per_proc_s, key=per_proc_s.get)
    dom_launch_s = per_proc_s[dom] / args.steps
    achieved = FLOP_EQ_PER_EVAL[dom] * n / dom_launch_s / 1e12
    # ncu DRAM bytes of one 1e7-pair launch, scaled to this launch's pairs
    # (the kernels read and write every pair once, so traffic grows in proportion)
    t7 = load_traffic().get(f"{dom}_fp64_1e7")
    traffic = t7 * n / 1e7 if t7 else None
    per_process = {name: {"evals_per_s": n * args.steps / t, "ms_per_launch": 1e3 * t / args.steps,
                          "flop_eq_tflops": FLOP_EQ_PER_EVAL[name] * n * args.steps / t / 1e12,
                          "hbm_gbs": BYTES_PER_EVAL * n * args.steps / t / 1e9}
                   for name, t in per_proc_s.items()}
    line = {
        "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded log-uniform K in [1e-3,1e6] GeV, nu in [1e-7,1], q = nu K",
        "config": config_dict(n, world),
        "roofline": {"bound": "fp64", "kernel": f"{dom} FP64", "achieved": achieved, "peak": peak,
                     "unit": "TFLOP/s", "frac": achieved / peak if peak else None,
                     "traffic": traffic,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of a 1e7-pair launch "
                                       "(profiles/traffic.json) x n / 1e7",
                     "peak_source": "FP64 FMA-chain probe (noa_dcs_probe_fma, libnoa_dcs_diag.so) measured in "
                                    "this run",
                     "numerator": f"{FLOP_EQ_PER_EVAL[dom]} flop-eq/eval x {n} evals per launch",
                     "convention": "flop-eq counted on the oracle, each libm log/exp/pow = 20; the kernels "
                                   "compute log/exp/reciprocal mostly on the integer and FP32 pipes (1/2/0 FP64 "
                                   "instructions), so frac can exceed 1; hw_view is the hardware roofline",
                     "hw_view": hw_view(dom)},
        "per_process": per_process,
        "variants": variants,
        "e2e": e2e,
        "clocks": clocks.summary(),
        "gpu_launches": 4 * args.steps,
    }
    if parity is not None:
        line["parity_vs_oracle"] = parity
    if ref_cuda is not None:
        line["reference_cuda_bremsstrahlung"] = ref_cuda
    if not args.no_batched:
        line["batched"] = time_batched(torch, args)
    if not args.no_integrals:
        line["recoil_integrals"] = time_integrals(torch, args, with_cpu=not args.no_cpu_baseline and world == 1)
        line["transport"] = time_transport(torch, args, with_cpu=not args.no_cpu_baseline and world == 1)
    if not args.no_surrogate:
        line["surrogate"] = time_surrogate(torch, args)
    if not args.no_cpu_baseline and world == 1:
        cb = cpu_reference_rate(min(n, 1_000_000))
        c1 = cpu_reference_rate(min(n, 100_000), reps=3, threads=1)
        what = ("the reference's own dcs::pvmap (src/noa/pms/dcs.hh compiled on this host with its benchmark's "
                "flags, -O3 -fopenmp)"
                if cb["kind"] == "reference" else "the CPU oracle port of dcs::pvmap (OpenMP)")
        line["cpu_baseline"] = {"value": cb["value"], "unit": "evals/s", "cores": cb["cores"], "kind": cb["kind"],
                                "sample": f"{what}: first 1e6 pairs of the workload, all four processes, "
                                          "median of 5 after a warm-up",
                                "per_process": cb["per_process"],
                                "single_thread": {"value": c1["value"], "per_process": c1["per_process"],
                                                  "sample": "dcs::vmap, first 1e5 pairs, median of 3"}}
    line["summary"] = summarise(line)
    print(json.dumps(line), flush=True)
    if world > 1:
        tdist.destroy_process_group()


def _r(x, d=4):
    """x rounded to d significant digits (None passes through)."""
    if x is None:
        return None
    return float(f"{x:.{d}g}")


def summarise(line):
    """A compact digest of the whole line, printed last so that a reader
    keeping only the end of the line still has every headline figure."""
    s = {"workload": line["config"]["workload"], "fp64_evals_per_s": _r(line["value"]),
         "e2e_evals_per_s": _r((line.get("e2e") or {}).get("value")),
         "roofline_frac": _r(line["roofline"]["frac"], 3),
         "fp64_pipe_frac": _r(((line["roofline"].get("hw_view") or {}).get("frac")), 3)}
    par = line.get("parity_vs_oracle")
    if par:
        s["fp64_vs_oracle"] = {k: {"mean": _r(v["mean_rel"], 2), "max": _r(v["max_rel"], 2),
                                   "cond_ratio": _r(v["cond_ratio"], 2), "zeros_equal": v["zero_pattern_equal"]}
                               for k, v in par.items() if isinstance(v, dict)}
    f = (line.get("variants") or {}).get("fp32c")
    if f:
        s["fp32c"] = {k: {"x_fp64": _r(v["speedup_vs_fp64"], 3), "max": _r(v["max_rel"], 2),
                          "median": _r(v["median_rel"], 2)} for k, v in f.items() if k in PROCESSES}
        s["fp32c"]["all"] = {"x_fp64": _r(f["all_processes"]["speedup_vs_fp64"], 3),
                             "evals_per_s": _r(f["all_processes"]["evals_per_s"])}
    rc = line.get("reference_cuda_bremsstrahlung")
    if rc:
        s["reference_cuda_brems"] = ({"ms": _r(rc["ms_per_launch"]), "ours_ms": _r(rc["ours_ms_per_launch"]),
                                      "x": _r(rc["speedup_of_ours"], 3),
                                      "mean_vs_ours": _r(rc["vs_ours"]["mean_rel"], 2)}
                                     if rc.get("available") else "unavailable")
    b = line.get("batched")
    if b:
        s["batched_evals_per_s"] = {p: _r(b[p]["all_processes"]["evals_per_s"]) for p in ("fp64", "fp32c")}
    sg = line.get("surrogate")
    if sg:
        s["surrogate"] = {k: {"x_fp64": _r(v["speedup_vs_fp64"], 3), "x_fp32c": _r(v["speedup_vs_fp32c"], 3),
                              "x_no_net": _r(v.get("speedup_vs_no_network"), 3),
                              "max": _r(v["max_rel"], 2), "above_1e-3": v["frac_above_1e-3"],
                              "net_share": _r(v["network_share_of_open"], 2),
                              "train_s": _r(v["training"].get("train_seconds"), 3)}
                          for k, v in sg.items() if isinstance(v, dict) and "speedup_vs_fp64" in v}
    cb = line.get("cpu_baseline")
    if cb:
        s["cpu_baseline"] = {"evals_per_s": _r(cb["value"]), "kind": cb["kind"], "cores": cb["cores"]}
    return s


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
