"""The float-first decisions of the FP64 kernels against the reference's exact
IEEE decisions, on pairs placed at every bound.

The kernels decide which pairs are open (pair production, dcs.hh:151-176;
photonuclear, dcs.hh:357-381), whether bremsstrahlung's electron term exists
(physics.hh:133, 142) and whether ionisation's first exit is taken
(dcs.hh:413-419) in float or lean arithmetic first, with a margin, and take
the reference's IEEE test only inside the margin.  noa_dcs_decision_check
(libnoa_dcs_diag.so) evaluates both on the device; here no pair may show a
disagreement.  Pairs: the seeded workload, and pairs within a few ulp to
1e-4 (relative) of each bound, located by bisection where a bound has no
closed form.
"""
import numpy as np
import pytest
import torch

from noa_gb300 import _lib
from noa_gb300.elements import ELEMENTS, MUON_MASS, STANDARD_ROCK
from noa_gb300.workload import kinetic_recoil

pytestmark = pytest.mark.gpu

ME = 0.51099895000e-3
M = MUON_MASS
SQRTE = 1.6487212707
ELS = [STANDARD_ROCK, ELEMENTS[1], ELEMENTS[82]]


def check(proc, K, q, el):
    lib = _lib.load_diag()
    tk = torch.from_numpy(np.ascontiguousarray(K, dtype=np.float64)).cuda()
    tq = torch.from_numpy(np.ascontiguousarray(q, dtype=np.float64)).cuda()
    out = torch.empty_like(tk)
    _lib.check(lib.noa_dcs_decision_check(proc, tk.data_ptr(), tq.data_ptr(), out.data_ptr(), tk.numel(),
                                          el.A, el.I, el.Z, M, None))
    torch.cuda.synchronize()
    return out.cpu().numpy()


def around(x, rng, rel=1e-4, ulps=8):
    """x moved by a few ulp and by relative amounts up to rel, both ways."""
    x = np.asarray(x, dtype=np.float64)
    steps = rng.integers(-ulps, ulps + 1, x.size)
    near = x + steps * np.spacing(x)
    far = x * (1 + rng.uniform(-rel, rel, x.size))
    return np.concatenate([x, near, far])


def bisect(f, lo, hi, iters=80):
    """Vectorised bisection for a sign change of f between lo and hi (f(lo) < 0 <= f(hi))."""
    lo, hi = lo.copy(), hi.copy()
    for _ in range(iters):
        mid = 0.5 * (lo + hi)
        neg = f(mid) < 0
        lo = np.where(neg, mid, lo)
        hi = np.where(neg, hi, mid)
    return hi


def log_uniform(rng, n, lo, hi):
    return np.exp(rng.uniform(np.log(lo), np.log(hi), n))


def assert_agree(codes, label, undecided_max=None):
    bad = int((codes == -2).sum())
    assert bad == 0, f"{label}: {bad} of {codes.size} fast decisions differ from the exact ones"
    if undecided_max is not None:
        assert float((codes == -1).mean()) <= undecided_max, (label, float((codes == -1).mean()))


@pytest.mark.parametrize("proc", range(4), ids=["bremsstrahlung", "pair_production", "photonuclear", "ionisation"])
def test_seeded_workload(cuda_device, proc):
    K, q = kinetic_recoil(2_000_000, offset=777)
    for el in ELS:
        codes = check(proc, K, q, el)
        assert_agree(codes, f"seeded {el.Z}", undecided_max=1e-4 if proc == 3 else None)


def test_bremsstrahlung_electron_term_edge(cuda_device):
    rng = np.random.default_rng(11)
    K = log_uniform(rng, 200_000, 1e-3, 1e6)
    E = K + M
    qe = E / (1. + 0.5 * M * M / (ME * E))  # physics.hh:133
    for el in ELS:
        Ka = np.tile(K, 3)
        assert_agree(check(0, Ka, around(qe, rng), el), f"qe_max Z={el.Z}")


def test_pair_production_bounds(cuda_device):
    rng = np.random.default_rng(12)
    for el in ELS:
        Z13 = el.Z ** (1. / 3.)
        shift = M * (1. - 0.75 * SQRTE * Z13)
        K = log_uniform(rng, 100_000, 1e-2, 1e6)
        K = K[K + shift > 4. * ME * 1.01]
        # q <= 4 me and q >= K + shift
        lo = around(np.full(K.size, 4. * ME), rng)
        hi = around(K + shift, rng)
        Ka = np.tile(K, 3)
        assert_agree(check(1, Ka, lo, el), f"4 me Z={el.Z}")
        assert_agree(check(1, Ka, hi, el), f"K + shift Z={el.Z}")

        # argmin = 1 (dcs.hh:169-176), the reference's formula in IEEE double:
        # interior crossings exist just above the lowest open K (x1 large);
        # scan a q grid per K
        # and bisect every sign change (argmin -> 1 as q -> 4 me is the 4 me
        # bound above)
        k_lo = 4. * ME * 1.01 - shift
        Ks = log_uniform(rng, 20_000, k_lo, 2. * k_lo)

        def argmin_minus_1(qq, KK):
            gamma = 1. + KK / M
            x0 = 4. * ME / qq
            x1 = 6. / (gamma * (gamma - qq / M))
            return (x0 + 2. * (1. - x0) * x1) / (1. + (1. - x1) * np.sqrt(1. - x0)) - 1.
        G = 256
        lq = np.log(4. * ME * 1.001) + (np.log(Ks + shift) - np.log(4. * ME * 1.001))[:, None] * np.linspace(0, 1, G)
        qg = np.exp(lq)
        qg[:, -1] = np.nextafter(Ks + shift, 0)
        with np.errstate(all="ignore"):
            fg = argmin_minus_1(qg, Ks[:, None])
            roots, kk = [], []
            for sgn in (1., -1.):  # rising and falling crossings
                g = sgn * fg
                cross = (g[:, :-1] < 0) & (g[:, 1:] >= 0)
                r, j = np.nonzero(cross)
                roots.append(bisect(lambda x: sgn * argmin_minus_1(x, Ks[r]), qg[r, j], qg[r, j + 1]))
                kk.append(Ks[r])
        qs, Kr = np.concatenate(roots), np.concatenate(kk)
        if el.Z != 82:  # lead's window has no interior crossing
            assert qs.size > 1000, (el.Z, qs.size)
        if qs.size:
            assert_agree(check(1, np.tile(Kr, 3), around(qs, rng), el), f"argmin = 1 Z={el.Z}")


def test_photonuclear_bounds(cuda_device):
    rng = np.random.default_rng(13)
    mpi, Mn = 0.134977, 0.931494
    q_min = mpi * (1.0 + 0.5 * mpi / Mn)
    for el in ELS:
        K = log_uniform(rng, 100_000, 1.0, 1e6)
        Ka = np.tile(K, 3)
        for label, edge in (("q = 1", np.ones(K.size)), ("q = 2e-3 K", 2e-3 * K), ("q = E - m", (K + M) - M),
                            ("q = q_min", np.full(K.size, q_min))):
            assert_agree(check(2, Ka, around(edge, rng), el), f"{label} Z={el.Z}")

        # (Q2max < Q2min, dcs.hh:377, closes nothing here: past the first exit
        # q >= 1 GeV, so Q2max = 2 M (q - mpi) - mpi^2 >= 1.59 GeV^2, while
        # Q2min = m^2 y^2 / (1 - y) stays below m (K + m) y^2 < Q2max up to q -> K.)


def test_ionisation_first_exit(cuda_device):
    rng = np.random.default_rng(14)

    def wmax(KK):
        P2 = KK * (KK + 2. * M)
        return 2. * ME * P2 / (M * M + ME * (ME + 2. * (KK + M)))
    K = log_uniform(rng, 200_000, 1e-3, 1e6)
    Ka = np.tile(K, 3)
    # K at the 5% threshold: W_max(K) = 0.05 K
    Kt = bisect(lambda KK: wmax(KK) - 0.05 * KK, np.full(1000, 1e-4), np.full(1000, 1e3))
    Kt = around(np.repeat(Kt[:1], 200_000), rng, rel=1e-4, ulps=64)
    for el in ELS:
        codes = check(3, Ka, around(wmax(K), rng), el)
        assert_agree(codes, f"q = W_max Z={el.Z}")
        assert float((codes >= 0).mean()) > 0.2  # outside the margin the float test decides
        assert_agree(check(3, Kt, 1e-3 * wmax(Kt), el), f"W_max = 5% K Z={el.Z}")


def test_special_inputs(cuda_device):
    K = np.array([np.nan, 1.0, np.inf, 0.0, 1.0, -1.0, 1e6, 1e-3, 1e30, 5e-324, 1.0, 1e-300])
    q = np.array([1.0, np.nan, 1.0, 1e-3, 0.0, 0.5, np.inf, 1e-3, 1e29, 1e-3, -0.5, 1e-301])
    for proc in range(4):
        assert_agree(check(proc, K, q, STANDARD_ROCK), f"special proc {proc}")


def test_decision_check_arguments(cuda_device):
    lib = _lib.load_diag()
    t = torch.zeros(4, dtype=torch.float64, device="cuda")
    host = np.zeros(4)
    args = (t.data_ptr(), t.data_ptr(), t.data_ptr(), 4, 22., 1.364e-7, 11, M, None)
    assert lib.noa_dcs_decision_check(4, *args) != 0
    assert lib.noa_dcs_decision_check(0, t.data_ptr(), t.data_ptr(), host.ctypes.data, 4, 22., 1.364e-7, 11, M,
                                      None) != 0
    assert lib.noa_dcs_decision_check(0, *args[:5], -1., 11, M, None) != 0
    assert lib.noa_dcs_decision_check(0, *args) == 0
