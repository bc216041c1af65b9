"""Comparison helpers shared by the parity tests."""
import numpy as np

PROCESSES = ("bremsstrahlung", "pair_production", "photonuclear", "ionisation")

# The FP64 gate: the reference's own relative_error metric (a mean,
# src/noa/utils/common.hh:228-236) at most 1e-12 per process.  Individual
# points may move more because this path's log/exp differ from glibc's by a
# few ulp and some points are ill-conditioned (the reference itself moves by
# up to ~1e-10 under 2-ulp input perturbations).  So each point is held to
# the reference's own conditioning there: its relative error at most
# COND_FACTOR times the largest relative change of the reference's output
# under +-COND_DELTA relative changes of K and q, plus COND_FLOOR.  MAX_REL
# caps every point in addition.
MEAN_REL_FP64 = 1e-12
MAX_REL_FP64 = 1e-8
COND_DELTA = 4e-16
COND_FACTOR = 64.0
COND_FLOOR = 1e-12


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


def conditioning(process, K, q, element, mass, expected=None):
    """Per point, the largest relative change of the oracle's (the
    reference's) output when K and q move by +-COND_DELTA relative, in the
    four sign combinations; 0 where the output is 0 or not finite."""
    import oracle
    K = np.asarray(K, dtype=np.float64)
    q = np.asarray(q, dtype=np.float64)
    e = oracle.dcs(process, K, q, element, mass) if expected is None else np.asarray(expected, np.float64)
    ok = np.isfinite(e) & (e != 0)
    sens = np.zeros_like(e)
    for dk in (COND_DELTA, -COND_DELTA):
        for dq in (COND_DELTA, -COND_DELTA):
            o = oracle.dcs(process, K * (1 + dk), q * (1 + dq), element, mass)
            with np.errstate(invalid="ignore", divide="ignore", over="ignore"):
                r = np.abs(o - e) / np.abs(e)
            r = np.where(ok & np.isfinite(r), r, np.where(ok, np.inf, 0.0))
            sens = np.maximum(sens, r)
    return sens


def assert_conditioned(computed, expected, sens, label="", factor=COND_FACTOR, floor=COND_FLOOR):
    """Every finite non-zero point within factor x sens + floor (relative)."""
    c = np.asarray(computed, dtype=np.float64)
    e = np.asarray(expected, dtype=np.float64)
    m = np.isfinite(c) & np.isfinite(e) & (e != 0)
    err = np.abs(c[m] - e[m]) / np.abs(e[m])
    bar = factor * sens[m] + floor
    bad = err > bar
    if bad.any():
        i = int(np.argmax(err - bar))
        raise AssertionError(f"{label}: {int(bad.sum())} points above {factor:g} x conditioning + {floor:g}; "
                             f"worst err {err[i]:.3e} vs bar {bar[i]:.3e} (sens {sens[m][i]:.3e})")


def assert_fp64_parity(computed, expected, label="", inputs=None):
    """The FP64 bar.  inputs = (process, K, q, element, mass) adds the
    per-point conditioning bar against the reference's own response."""
    s = rel_stats(computed, expected)
    assert s["nonfinite_agree"], f"{label}: NaN/inf pattern differs {s}"
    assert s["zero_agree"], f"{label}: zero pattern differs {s}"
    assert s["mean"] <= MEAN_REL_FP64, f"{label}: mean relative error {s}"
    assert s["max"] <= MAX_REL_FP64, f"{label}: max relative error {s}"
    if inputs is not None:
        process, K, q, element, mass = inputs
        assert_conditioned(computed, expected, conditioning(process, K, q, element, mass, expected), label)
    return s
