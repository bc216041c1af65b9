"""CPU checks of bench.py's contract: the flop numerator re-derived from the
oracle's operation count, and the reference arm's JSON line."""
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
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["value"] == d["value"]
    assert d["metric"] == bench.METRIC and d["higher_is_better"] is True
