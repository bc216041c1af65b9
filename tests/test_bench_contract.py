"""CPU checks of bench.py's contract: the flop numerator re-derived from the
oracle's operation count, the reference arm's JSON line, and the summary
digest printed last on the line."""
import json
import subprocess
import sys

import numpy as np

import bench
import oracle
from noa_gb300.elements import MUON_MASS, STANDARD_ROCK
from noa_gb300.workload import kinetic_recoil


def test_flop_equivalents_match_the_oracle_count(built):
    K, q = kinetic_recoil(200_000)
    for p, name in enumerate(bench.PROCESSES):
        c = oracle.opcount(p, K, q, STANDARD_ROCK, MUON_MASS)
        per = (c["add"] + c["mul"] + c["div"] + c["sqrt"] + c["cmp"] + 20 * c["trans"]) / len(K)
        assert abs(per - bench.FLOP_EQ_PER_EVAL[name]) <= 0.01 * bench.FLOP_EQ_PER_EVAL[name], (name, per)


def test_reference_arm_prints_one_json_line(built):
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0",
                        "--n", "20000"], capture_output=True, text=True, cwd=bench.ROOT, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = [x for x in r.stdout.splitlines() if x.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "evals/s" and d["value"] > 0
    # the reference's own dcs::pvmap where oracle/build_ref.sh compiled it, else the port
    assert d["cpu_baseline"]["kind"] == ("reference" if oracle.ref_available() else "port")
    assert d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["value"] == d["value"]
    assert d["metric"] == bench.METRIC and d["higher_is_better"] is True


def test_summary_is_last_and_compact():
    """summarise() on a line shaped like the GPU arm's, with every optional
    section present: the digest stays a few kB and is the line's last key."""
    per = {p: {"evals_per_s": 1e9, "ms_per_launch": 1.0, "speedup_vs_fp64": 10.0, "max_rel": 9e-7,
               "median_rel": 5e-8, "mean_rel": 6e-8, "zero_pattern_equal": True} for p in bench.PROCESSES}
    per["all_processes"] = {"evals_per_s": 2e10, "speedup_vs_fp64": 12.0}
    line = {"value": 1.6e9, "config": bench.config_dict(100_000_000, 1), "e2e": {"value": 1.5e9},
            "roofline": {"frac": 0.7}, "variants": {"fp32c": per},
            "parity_vs_oracle": {"sample": "x", **{p: {"mean_rel": 1e-15, "max_rel": 1e-11, "cond_ratio": 0.01,
                                                       "zero_pattern_equal": True} for p in bench.PROCESSES}},
            "reference_cuda_bremsstrahlung": {"available": True, "ms_per_launch": 30.0, "ours_ms_per_launch": 13.6,
                                              "speedup_of_ours": 2.2, "vs_ours": {"mean_rel": 1e-16}},
            "batched": {"fp64": {"all_processes": {"evals_per_s": 1.6e9}},
                        "fp32c": {"all_processes": {"evals_per_s": 1.5e10}}},
            "surrogate": {"error_bound": 1e-3, **{p: {"speedup_vs_fp64": 11.0, "speedup_vs_fp32c": 1.3,
                                                      "max_rel": 5e-4, "frac_above_1e-3": 0.0,
                                                      "network_share_of_open": 0.3,
                                                      "training": {"train_seconds": 30.0}}
                                                  for p in ("pair_production", "photonuclear")}},
            "cpu_baseline": {"value": 1e8, "kind": "reference", "cores": 16}}
    line["summary"] = bench.summarise(line)
    text = json.dumps(line)
    assert list(json.loads(text))[-1] == "summary"
    assert len(json.dumps(line["summary"])) < 2500


def test_hardware_roofline_view():
    """roofline.hw_view: ncu's pipe utilisations of each FP64 kernel, from the
    committed capture summary (profiles/traffic.json), the FP64 pipe as the
    bound; the summary carries its fraction."""
    for p in bench.PROCESSES:
        hw = bench.hw_view(p)
        assert hw is not None and hw["bound"] == "fp64 pipe", p
        assert 0.0 < hw["frac"] <= 1.0 and hw["frac"] == hw["pipes"]["fp64_pipe"]
        assert set(hw["pipes"]) == {"fp64_pipe", "alu_pipe", "fma_pipe", "issue"}
        assert "profiles/" in hw["source"]
    assert bench.hw_view("no such process") is None
    line = {"value": 2.8e9, "config": bench.config_dict(100_000_000, 1), "e2e": None,
            "roofline": {"frac": 1.16, "hw_view": bench.hw_view("pair_production")}}
    s = bench.summarise(line)
    assert s["fp64_pipe_frac"] == round(bench.hw_view("pair_production")["frac"], 3)
