"""GPU tests of the C++/LibTorch drop-in (include/noa_gb300/dcs_cuda.hh,
noa::pms::dcs::cuda::{vmap,map}_<process>) through the Python module that
mirrors the reference notebook's muons_cuda extension."""
import numpy as np
import pytest
import torch

import oracle
from noa_gb300.elements import ELEMENTS, MUON_MASS, STANDARD_ROCK
from noa_gb300.workload import kinetic_recoil
from tests.parity import PROCESSES, assert_fp64_parity, same_bits

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def muons_cuda(cuda_device):
    from noa_gb300 import _muons_cuda
    return _muons_cuda


@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
def test_notebook_style_call(muons_cuda, process):
    """docs/pms/muon_dcs_calc.ipynb: linspace energies, q = 0.0505 K, standard rock."""
    K = torch.linspace(1e-3, 1e6, 10000).double()
    q = 0.0505 * K
    got = getattr(muons_cuda, PROCESSES[process])(K.cuda(), q.cuda()).cpu().numpy()
    exp = oracle.dcs(process, K.numpy(), q.numpy(), STANDARD_ROCK, MUON_MASS)
    assert_fp64_parity(got, exp, PROCESSES[process], inputs=(process, K.numpy(), q.numpy(), STANDARD_ROCK, MUON_MASS))


def test_notebook_cpu_gpu_agreement_like_the_reference(muons_cuda):
    """The notebook prints sum|brems_cpu - brems_gpu| = 3.29e-18 over its 10000 pairs."""
    K = torch.linspace(1e-3, 1e6, 10000).double()
    q = 0.0505 * K
    got = muons_cuda.bremsstrahlung(K.cuda(), q.cuda()).cpu().numpy()
    exp = oracle.dcs(0, K.numpy(), q.numpy(), STANDARD_ROCK, MUON_MASS)
    assert np.abs(got - exp).sum() < 1e-15


@pytest.mark.parametrize("process", range(4), ids=PROCESSES)
def test_drop_in_equals_c_abi(muons_cuda, process):
    from noa_gb300 import dcs
    K, q = kinetic_recoil(100000, offset=31337)
    tk, tq = torch.from_numpy(K).cuda(), torch.from_numpy(q).cuda()
    el = ELEMENTS[26]
    a = getattr(muons_cuda, PROCESSES[process])(tk, tq, el.A, el.I, el.Z, MUON_MASS)
    b = dcs.map(process, tk, tq, el, MUON_MASS)
    r = torch.empty_like(tk)
    muons_cuda.vmap(process, 0, r, tk, tq, el.A, el.I, el.Z, MUON_MASS)
    torch.cuda.synchronize()
    assert same_bits(a.cpu().numpy(), b.cpu().numpy())
    assert same_bits(r.cpu().numpy(), b.cpu().numpy())


def test_drop_in_errors_are_c10_errors(muons_cuda):
    d = torch.zeros(8, dtype=torch.float64, device="cuda")
    with pytest.raises(RuntimeError, match="Double"):
        muons_cuda.bremsstrahlung(d.float(), d)
    with pytest.raises(RuntimeError, match="CUDA"):
        muons_cuda.bremsstrahlung(d.cpu(), d.cpu())
    with pytest.raises(RuntimeError, match="size mismatch"):
        muons_cuda.vmap(0, 0, d[:4], d, d)
    with pytest.raises(RuntimeError, match="contiguous"):
        muons_cuda.vmap(0, 0, d[::2], d[::2].contiguous(), d[::2].contiguous())
    with pytest.raises(RuntimeError, match="invalid element"):
        muons_cuda.bremsstrahlung(d, d, 22.0, 1e-7, 0)


def test_per_k_functions_through_the_drop_in(muons_cuda):
    """recoil_integral, soft_scattering and the Coulomb chain through the
    LibTorch layer, with the reference's argument order, against the oracle."""
    K, _ = kinetic_recoil(3000, offset=123)
    tk = torch.from_numpy(K).cuda()
    out = torch.empty_like(tk)
    muons_cuda.recoil_integral(1, 0, out, tk)
    assert_fp64_parity(out.cpu().numpy(), oracle.recoil_integral(1, 0, K, 0.05, STANDARD_ROCK, MUON_MASS, 180),
                       "recoil integral")
    muons_cuda.soft_scattering(out, tk)
    assert_fp64_parity(out.cpu().numpy(), oracle.soft_scattering(K, STANDARD_ROCK, MUON_MASS), "soft scattering")
    n = K.size
    f64 = dict(dtype=torch.float64, device="cuda")
    fCM, screen, fspin, invlambda = (torch.zeros(n, 2, **f64), torch.zeros(n, 9, **f64), torch.zeros(n, **f64),
                                     torch.zeros(n, **f64))
    muons_cuda.coulomb_data(fCM, screen, fspin, invlambda, tk)
    G = torch.zeros(n, 2, **f64)
    muons_cuda.coulomb_transport(G, screen, fspin, torch.tensor(1.0, **f64))
    mu0, lb_h = torch.zeros(n, **f64), torch.zeros(n, **f64)
    muons_cuda.hard_scattering(mu0, lb_h, G.view(1, n, 2), fCM.view(1, n, 2), screen.view(1, n, 9),
                               invlambda.view(1, n), fspin.view(1, n))
    e = oracle.coulomb_data(K, STANDARD_ROCK, MUON_MASS)
    eG = oracle.coulomb_transport(e[1], e[2], 1.0)
    e_mu0, e_lb_h = oracle.hard_scattering(eG, e[0], e[1], e[3], e[2])
    assert_fp64_parity(mu0.cpu().numpy(), e_mu0, "mu0")
    assert_fp64_parity(lb_h.cpu().numpy(), e_lb_h, "lb_h")
    with pytest.raises(RuntimeError):
        muons_cuda.coulomb_transport(G, screen, fspin, torch.zeros(5, **f64))
