"""Generates tests/golden/dcs_golden.npz from the REFERENCE's own code.

Run where a grinisrit/noa checkout exists, naming it by argument or by the
NOA_CHECKOUT environment variable:

    python tests/golden/make_golden.py NOA_CHECKOUT

It compiles the unmodified src/noa/pms/dcs.hh behind oracle/ref_dcs_wrapper.cc
(oracle/build_ref.sh), evaluates it through the reference's dcs::vmap and
dcs::vmap_integral(dcs::recoil_integral(...)) on

  * seeded pairs of the benchmark law (noa_gb300.workload, seed 987654),
  * the notebook inputs of docs/pms/muon_dcs_calc.ipynb (cell "linspace"):
    K = float32 linspace(1e-3, 1e6, 10000) cast to float64, q = 0.0505 K
    (its first 64 points and every 50th after them),
  * hand-placed edge cases at every early return of the four processes,
  * three elements: standard rock (the reference's only element), hydrogen
    (the Z == 1 branches) and lead,

and stores inputs and outputs.  The fixtures pin the CPU oracle (bit for bit)
and the CUDA kernels (to the stated tolerance) on hosts without the checkout.

A second file, elastic_golden.npz, holds the reference's elastic-scattering
and transverse-transport outputs (dcs::coulomb_data, coulomb_transport,
hard_scattering, soft_scattering, dcs.hh:499-952) on a log grid of kinetic
energies, seeded energies and the kinematic edges of those functions, for the
same three elements, plus hard scattering over the three elements at once.
"""
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from noa_gb300.elements import ELEMENTS, ELECTRON_MASS, MUON_MASS, STANDARD_ROCK, X_FRACTION  # noqa: E402
from noa_gb300.workload import kinetic_recoil  # noqa: E402

GOLDEN_ELEMENTS = {"rock": STANDARD_ROCK, "hydrogen": ELEMENTS[1], "lead": ELEMENTS[82]}
N_SEEDED = 2048
N_INTEGRAL = 128


def edge_cases():
    """(K, q) pairs placed on the early returns of dcs.hh / physics.hh."""
    me, m = ELECTRON_MASS, MUON_MASS
    Ks = [1e-3, 5e-3, 0.05, 0.1, 1.0, 3.7, 10.0, 50.0, 1e3, 1e5, 1e6]
    K, q = [], []
    for k in Ks:
        E = k + m
        P2 = k * (k + 2 * m)
        wmax = 2.0 * me * P2 / (m * m + me * (me + 2.0 * E))
        qe_max = E / (1.0 + 0.5 * m * m / (me * E))
        for v in (4 * me, np.nextafter(4 * me, 1), np.nextafter(4 * me, 0),   # pair production lower cut
                  k, np.nextafter(k, 0), np.nextafter(k, 2 * k + 1),          # q -> K
                  1.0, np.nextafter(1.0, 0), 2e-3 * k,                        # photonuclear cuts
                  wmax, np.nextafter(wmax, 0), np.nextafter(wmax, 1e9),       # ionisation W_max
                  qe_max, np.nextafter(qe_max, 0),                            # bremsstrahlung qe_max
                  0.62 * STANDARD_ROCK.I, 1e-10, 1e-7 * k, 0.5 * k, 0.99 * k, 0.999999 * k):
            K.append(k)
            q.append(float(v))
    # pair production upper bound q = K + m (1 - 0.75 sqrte Z^1/3) for standard rock
    z13 = 11 ** (1.0 / 3.0)
    for k in Ks:
        qmax = k + m * (1.0 - 0.75 * 1.6487212707 * z13)
        for v in (qmax, np.nextafter(qmax, 0), np.nextafter(qmax, 1e9)):
            K.append(k)
            q.append(float(v))
    # ionisation radiative-correction threshold K = 0.5 (m - me)^2 / me
    kr = 0.5 * (m - me) ** 2 / me
    for k in (kr, np.nextafter(kr, 0), np.nextafter(kr, 1e9)):
        for v in (1e-4, 1e-3, 0.01):
            K.append(float(k))
            q.append(v)
    # special values (IEEE propagation must match the CPU)
    for k, v in ((1.0, 0.0), (0.0, 1e-3), (np.nan, 1.0), (1.0, np.nan), (np.inf, 1.0), (10.0, -1.0)):
        K.append(k)
        q.append(v)
    return np.array(K, dtype=np.float64), np.array(q, dtype=np.float64)


def main():
    noa = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("NOA_CHECKOUT")
    if not noa or not os.path.exists(os.path.join(noa, "src", "noa", "pms", "dcs.hh")):
        sys.exit("make_golden.py: name a grinisrit/noa checkout (argument or NOA_CHECKOUT)")
    subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_ref.sh"), "all"], check=True,
                   env={**os.environ, "NOA_CHECKOUT": noa})
    out = {}
    Ks, qs = kinetic_recoil(N_SEEDED)
    import torch
    Kn = torch.linspace(1e-3, 1e6, 10000).double().numpy()
    Kn = np.concatenate([Kn[:64], Kn[64::50]])   # the printed head plus a stride of the rest
    qn = 0.0505 * Kn
    Ke, qe = edge_cases()
    out["seeded_K"], out["seeded_q"] = Ks, qs
    out["notebook_K"], out["notebook_q"] = Kn, qn
    out["edge_K"], out["edge_q"] = Ke, qe
    for ename, el in GOLDEN_ELEMENTS.items():
        for p, pname in enumerate(("bremsstrahlung", "pair_production", "photonuclear", "ionisation")):
            for sname, (K, q) in (("seeded", (Ks, qs)), ("notebook", (Kn, qn)), ("edge", (Ke, qe))):
                if sname == "notebook" and ename != "rock":
                    continue
                out[f"{sname}_{ename}_{pname}"] = oracle.ref_dcs(p, K, q, el, MUON_MASS)
    Ki = Ks[:N_INTEGRAL]
    out["integral_K"] = Ki
    for p, pname in enumerate(("bremsstrahlung", "pair_production", "photonuclear", "ionisation")):
        for moment, mname in ((0, "del"), (1, "cel")):
            out[f"integral_rock_{pname}_{mname}"] = oracle.ref_recoil_integral(
                p, moment, Ki, X_FRACTION, STANDARD_ROCK, MUON_MASS, 180)
    meta = {"mass": MUON_MASS, "xlow": X_FRACTION, "min_points": 180, "seed": 987654,
            "elements": {k: [v.A, v.I, v.Z] for k, v in GOLDEN_ELEMENTS.items()},
            "source": "reference src/noa/pms/dcs.hh via oracle/ref_dcs_wrapper.cc"}
    out["meta"] = np.array(json.dumps(meta))
    path = os.path.join(HERE, "dcs_golden.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes", len(out), "arrays")


def elastic_energies():
    """Kinetic energies for the elastic fixtures: a log grid over
    [1e-6, 1e6] GeV, seeded energies, and points around the switches of
    coulomb_screening_parameters (zeta2 = 1 moves with Z and K)."""
    grid = np.logspace(-6, 6, 193)
    seeded, _ = kinetic_recoil(N_INTEGRAL, offset=N_SEEDED)
    return np.concatenate([grid, seeded, [1e-9, 1e-7, 0.1, 0.2, 0.5]])


def elastic():
    out = {}
    K = elastic_energies()
    out["K"] = K
    mu_var = np.logspace(-25, 0, K.size)
    stack = {name: [] for name in ("fCM", "screen", "fspin", "invlambda", "G")}
    for ename, el in GOLDEN_ELEMENTS.items():
        fCM, screen, fspin, invlambda = oracle.ref_coulomb_data(K, el, MUON_MASS)
        out[f"{ename}_fCM"], out[f"{ename}_screen"] = fCM, screen
        out[f"{ename}_fspin"], out[f"{ename}_invlambda"] = fspin, invlambda
        G = oracle.ref_coulomb_transport(screen, fspin, 1.0)
        out[f"{ename}_G"] = G
        out[f"{ename}_G_mu"] = oracle.ref_coulomb_transport(screen, fspin, mu_var)
        out[f"{ename}_mu0"], out[f"{ename}_lb_h"] = oracle.ref_hard_scattering(G, fCM, screen, invlambda, fspin)
        out[f"{ename}_soft"] = oracle.ref_soft_scattering(K, el, MUON_MASS)
        for name, v in zip(("fCM", "screen", "fspin", "invlambda", "G"), (fCM, screen, fspin, invlambda, G)):
            stack[name].append(v)
    st = {k: np.stack(v) for k, v in stack.items()}
    out["all_mu0"], out["all_lb_h"] = oracle.ref_hard_scattering(st["G"], st["fCM"], st["screen"],
                                                                 st["invlambda"], st["fspin"])
    out["mu_var"] = mu_var
    out["meta"] = np.array(json.dumps({"mass": MUON_MASS, "elements": list(GOLDEN_ELEMENTS),
                                       "source": "reference src/noa/pms/dcs.hh via oracle/ref_dcs_wrapper.cc"}))
    path = os.path.join(HERE, "elastic_golden.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes", len(out), "arrays")


if __name__ == "__main__":
    main()
    elastic()
