"""CPU tests of the oracle: pinned bit for bit to the reference's own outputs
(tests/golden, generated by tests/golden/make_golden.py from the unmodified
src/noa/pms/dcs.hh), to the notebook's printed values, and, where the
reference was compiled on this host, to fresh reference runs."""
import json

import numpy as np
import pytest

import oracle
from noa_gb300.elements import ELEMENTS, MUON_MASS, STANDARD_ROCK, X_FRACTION, AtomicElement
from noa_gb300.workload import kinetic_recoil
from tests.parity import PROCESSES, same_bits, same_or_both_nan


def _elements(golden):
    meta = json.loads(str(golden["meta"]))
    return {k: AtomicElement(*v) for k, v in meta["elements"].items()}


@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
@pytest.mark.parametrize("subset", ["seeded", "notebook", "edge"])
def test_oracle_matches_reference_golden(built, golden, process, subset):
    for ename, el in _elements(golden).items():
        key = f"{subset}_{ename}_{PROCESSES[process]}"
        if key not in golden:
            continue
        got = oracle.dcs(process, golden[f"{subset}_K"], golden[f"{subset}_q"], el, MUON_MASS, threads=1)
        exp = golden[key]
        if subset == "edge":
            assert same_or_both_nan(got, exp), key
            fin = np.isfinite(exp)
            assert same_bits(got[fin], exp[fin]), key
        else:
            assert same_bits(got, exp), key


# docs/pms/muon_dcs_calc.ipynb, outputs printed for the first five notebook pairs.
NOTEBOOK_KAT = {
    0: [3.5293e-04, 3.9395e-06, 4.0777e-06, 4.1341e-06, 4.1650e-06],
    1: [0.0, 6.5366e-06, 7.3699e-06, 7.7919e-06, 8.0572e-06],
    2: [0.0, 2.2912e-06, 2.1304e-06, 2.0719e-06, 2.0427e-06],
    3: [0.0, 3.0168e-05, 1.5300e-05, 1.0284e-05, 7.7575e-06],
}


@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
def test_oracle_notebook_known_answers(built, golden, process):
    got = oracle.dcs(process, golden["notebook_K"][:5], golden["notebook_q"][:5], STANDARD_ROCK, MUON_MASS)
    np.testing.assert_allclose(got, NOTEBOOK_KAT[process], rtol=5e-5, atol=0)


@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
@pytest.mark.parametrize("moment", [0, 1], ids=["del", "cel"])
def test_oracle_recoil_integrals_match_reference(built, golden, process, moment):
    key = f"integral_rock_{PROCESSES[process]}_{['del', 'cel'][moment]}"
    got = oracle.recoil_integral(process, moment, golden["integral_K"], X_FRACTION, STANDARD_ROCK, MUON_MASS,
                                 180, threads=1)
    assert same_bits(got, golden[key]), key


@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
def test_oracle_serial_equals_openmp(built, process):
    """dcs::vmap and dcs::pvmap are bit-identical in the reference; so here."""
    K, q = kinetic_recoil(20000, offset=5000)
    a = oracle.dcs(process, K, q, ELEMENTS[26], MUON_MASS, threads=1)
    b = oracle.dcs(process, K, q, ELEMENTS[26], MUON_MASS, threads=0)
    assert same_bits(a, b)


@pytest.mark.skipif(not oracle.ref_available(), reason="reference not compiled on this host")
@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
@pytest.mark.parametrize("z", [1, 8, 11, 26, 82])
def test_oracle_matches_compiled_reference(built, process, z):
    """Bit for bit against the reference compiled without FMA contraction
    (the build that made the goldens, on any host)."""
    K, q = kinetic_recoil(50000, offset=123456)
    el = ELEMENTS[z]
    assert same_bits(oracle.dcs(process, K, q, el, MUON_MASS), oracle.ref_dcs(process, K, q, el, MUON_MASS))


@pytest.mark.skipif(not oracle.ref_available("bench"), reason="reference not compiled on this host")
@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
@pytest.mark.parametrize("z", [1, 11, 82])
def test_benchmark_build_of_the_reference_meets_the_fp64_bar(built, process, z):
    """The timed CPU baseline is the reference built with its benchmark's
    flags; where the compiler fuses a*b + c (aarch64) its last bits move, so
    it is held to the FP64 bar (mean, per-point conditioning, zero pattern)
    against the oracle, and it runs dcs::pvmap and dcs::vmap identically."""
    from tests.parity import assert_fp64_parity
    K, q = kinetic_recoil(50000, offset=654321)
    el = ELEMENTS[z]
    got = oracle.ref_dcs(process, K, q, el, MUON_MASS, parallel=True, build="bench")
    assert same_bits(got, oracle.ref_dcs(process, K, q, el, MUON_MASS, parallel=False, build="bench"))
    assert_fp64_parity(got, oracle.dcs(process, K, q, el, MUON_MASS), f"{PROCESSES[process]} Z={z}",
                       inputs=(process, K, q, el, MUON_MASS))


@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
def test_opcount_runs_the_same_arithmetic(built, process):
    K, q = kinetic_recoil(2000, offset=77)
    c = oracle.opcount(process, K, q, STANDARD_ROCK, MUON_MASS)
    assert c["add"] > 0 and c["mul"] > 0
    # the counting scalar evaluates the same expressions: checksums agree
    ref = oracle.dcs(process, K, q, STANDARD_ROCK, MUON_MASS, threads=1)
    c2 = np.zeros(6)
    chk = oracle.lib().oracle_dcs_opcount(process, oracle._ptr(K), oracle._ptr(q), K.size, STANDARD_ROCK.A,
                                          STANDARD_ROCK.I, STANDARD_ROCK.Z, MUON_MASS, oracle._ptr(c2))
    seq = 0.0
    for v in ref.tolist():  # the C loop sums sequentially
        seq += v
    assert chk == seq


def test_relative_error_matches_reference_definition():
    c = np.array([1.0, 2.0, 0.0])
    e = np.array([1.0, 1.0, 0.0])
    assert oracle.relative_error(c, e) == pytest.approx((0 + 0.5 + 0) / 3)
