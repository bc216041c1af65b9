"""Comparison helpers shared by the parity tests."""
import numpy as np

PROCESSES = ("bremsstrahlung", "pair_production", "photonuclear", "ionisation")

# The FP64 gate: the reference's own relative_error metric (a mean,
# src/noa/utils/common.hh:228-236) at most 1e-12 per process.  Individual
# points may move more because CUDA's and glibc's log/exp/pow differ by an ulp
# and a few points are ill-conditioned (the reference itself moves by up to
# ~1e-10 under 2-ulp input perturbations); MAX_REL bounds those.
MEAN_REL_FP64 = 1e-12
MAX_REL_FP64 = 1e-8


def same_bits(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


def same_or_both_nan(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nan = np.isnan(a) & np.isnan(b)
    return bool(np.all(nan | (a == b)))


def rel_stats(computed, expected):
    """Mean (the reference metric), median, p99 and max relative error, over
    the finite entries, plus the zero / non-finite pattern agreement."""
    c = np.asarray(computed, dtype=np.float64)
    e = np.asarray(expected, dtype=np.float64)
    fin = np.isfinite(c) & np.isfinite(e)
    nonfinite_agree = bool(np.all(np.isfinite(c) == np.isfinite(e))) and same_or_both_nan(c[~fin], e[~fin])
    cf, ef = c[fin], e[fin]
    zero_agree = bool(np.all((cf == 0) == (ef == 0)))
    r = np.abs((cf - ef) / (cf + np.finfo(np.float64).tiny))
    nz = ef != 0
    rn = r[nz] if nz.any() else np.zeros(1)
    return {
        "mean": float(r.mean()) if r.size else 0.0,
        "median": float(np.median(rn)),
        "p99": float(np.quantile(rn, 0.99)),
        "max": float(rn.max()),
        "above_1e-12": int((rn > 1e-12).sum()),
        "zero_agree": zero_agree,
        "nonfinite_agree": nonfinite_agree,
        "n": int(c.size),
    }


def assert_fp64_parity(computed, expected, label=""):
    s = rel_stats(computed, expected)
    assert s["nonfinite_agree"], f"{label}: NaN/inf pattern differs {s}"
    assert s["zero_agree"], f"{label}: zero pattern differs {s}"
    assert s["mean"] <= MEAN_REL_FP64, f"{label}: mean relative error {s}"
    assert s["max"] <= MAX_REL_FP64, f"{label}: max relative error {s}"
    return s
