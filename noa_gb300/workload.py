"""Seeded synthetic (K, q) workloads for the muon DCS path.

The reference benchmarks (benchmark/measure-dcs-calc.hh:12-93) read PUMAS
golden energies that are fetched over the network; here every workload is a
counter-based stream so that the same pairs can be regenerated bit for bit on
any host: element i of stream s is splitmix64(seed + (2*i + s + 1) * golden)
mapped to a double in [0, 1).

Distribution (the reference's utils::SEED = 987654, common.hh:55):
    K  = 10 ** (9 u0 - 3)       log-uniform in [1e-3, 1e6] GeV
    nu = 10 ** (7 u1 - 7)       log-uniform in [1e-7, 1]
    q  = nu * K
"""
import numpy as np

SEED = 987654
_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def _mix(z):
    z = (z ^ (z >> np.uint64(30))) * _M1
    z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


def uniform(seed, stream, offset, n):
    """n doubles in [0, 1) from stream `stream` (0 or 1), starting at element `offset`."""
    idx = np.arange(offset, offset + n, dtype=np.uint64)
    with np.errstate(over="ignore"):
        state = np.uint64(seed) + (np.uint64(2) * idx + np.uint64(stream) + np.uint64(1)) * _GOLDEN
        bits = _mix(state) >> np.uint64(11)
    return bits.astype(np.float64) * (1.0 / 9007199254740992.0)


def kinetic_recoil(n, seed=SEED, offset=0, chunk=1 << 22):
    """Returns (K, q) float64 arrays of length n from the seeded log-uniform law."""
    K = np.empty(n, dtype=np.float64)
    q = np.empty(n, dtype=np.float64)
    for s in range(0, n, chunk):
        m = min(chunk, n - s)
        u0 = uniform(seed, 0, offset + s, m)
        u1 = uniform(seed, 1, offset + s, m)
        k = np.power(10.0, 9.0 * u0 - 3.0)
        K[s:s + m] = k
        q[s:s + m] = np.power(10.0, 7.0 * u1 - 7.0) * k
    return K, q


def element_counts(n_elements=10, lo=1e4, hi=3e7, seed=SEED):
    """Uneven per-element query counts, log-uniform in [lo, hi] (rounded)."""
    u = uniform(seed + 1, 0, 0, n_elements)
    return np.rint(np.power(10.0, u * np.log10(hi / lo) + np.log10(lo))).astype(np.int64)
