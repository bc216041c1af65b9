"""GPU tests of the learned surrogate's training path: the forward / backward
tensor-core kernels against CPU FP64 autograd of the same network, the
training data against the oracle, a short training run, and checkpoints."""
import numpy as np
import pytest
import torch

import oracle
from noa_gb300.elements import BATCH_Z, ELEMENTS, MUON_MASS
from noa_gb300.surrogate import NPARAM, Surrogate, init_params, training_pairs

pytestmark = pytest.mark.gpu

H = 128


def torch_reference(params, X, T):
    """The surrogate network in FP64 on the CPU (W2, W3 as the BF16 hi + lo
    pairs the tensor cores see); returns loss and gradient."""
    p = torch.tensor(params, dtype=torch.float64, requires_grad=True)
    o = 0

    def take(*shape):
        nonlocal o
        n = int(np.prod(shape))
        t = p[o:o + n].reshape(shape)
        o += n
        return t

    W1, b1, W2, b2, W3, b3, Wo, bo = take(H, 4), take(H), take(H, H), take(H), take(H, H), take(H), take(H), take(1)
    def bf(w):  # BF16 hi + lo pair as the tensor cores see it (straight-through)
        wd = w.detach()
        hi = wd.to(torch.bfloat16).to(torch.float64)
        lo = (wd.float() - hi.float()).to(torch.bfloat16).to(torch.float64)
        return w + (hi + lo - wd)
    x = torch.tensor(X, dtype=torch.float64)
    h1 = torch.nn.functional.silu(x @ W1.T + b1)
    h2 = torch.nn.functional.silu(h1 @ bf(W2).T + b2)
    h3 = torch.nn.functional.silu(h2 @ bf(W3).T + b3)
    y = h3 @ Wo + bo
    loss = ((y - torch.tensor(T, dtype=torch.float64)) ** 2).mean()
    loss.backward()
    return float(loss.detach()), p.grad.numpy()


BLOCKS = {"W1": (0, 512), "b1": (512, 640), "W2": (640, 17024), "b2": (17024, 17152), "W3": (17152, 33536),
          "b3": (33536, 33664), "Wo": (33664, 33792), "bo": (33792, 33793)}


@pytest.mark.parametrize("process", [1, 2])
def test_gradient_matches_cpu_autograd(cuda_device, process):
    rng = np.random.default_rng(3)
    params = init_params(seed=5)
    params[33664:33792] *= 10  # make every layer's gradient non-trivial
    n = 384
    X = rng.uniform(-1, 1, (n, 4)).astype(np.float32)
    T = rng.normal(0, 1, n).astype(np.float32)
    s = Surrogate(process, batch=512)
    s.set_params(params, np.zeros(10, np.float32))
    g, loss = s.gradient(torch.from_numpy(X).cuda(), torch.from_numpy(T).cuda())
    ref_loss, ref_g = torch_reference(params, X, T)
    g = g.cpu().numpy().astype(np.float64)
    assert abs(loss - ref_loss) <= 1e-4 * abs(ref_loss)
    for name, (a, b) in BLOCKS.items():
        d, r = g[a:b], ref_g[a:b]
        rel = np.linalg.norm(d - r) / max(np.linalg.norm(r), 1e-30)
        cos = float(d @ r / max(np.linalg.norm(d) * np.linalg.norm(r), 1e-30))
        # BF16 gradient operands: about 2^-8 per element, averaged
        assert rel < 2e-2 and cos > 0.9998, (name, rel, cos)


def test_prediction_matches_cpu_forward(cuda_device):
    rng = np.random.default_rng(4)
    params = init_params(seed=6)
    X = rng.uniform(-1, 1, (1000, 4)).astype(np.float32)
    s = Surrogate(1, batch=512)
    s.set_params(params, np.zeros(10, np.float32))
    got = s.predict(torch.from_numpy(X).cuda()).cpu().numpy()
    p = torch.tensor(params, dtype=torch.float64)
    W1, b1 = p[:512].reshape(H, 4), p[512:640]
    def hilo(w):
        hi = w.to(torch.bfloat16).double()
        return hi + (w.float() - hi.float()).to(torch.bfloat16).double()
    W2, b2 = hilo(p[640:17024].reshape(H, H)), p[17024:17152]
    W3, b3 = hilo(p[17152:33536].reshape(H, H)), p[33536:33664]
    Wo, bo = p[33664:33792], p[33792]
    silu = torch.nn.functional.silu
    y = silu(silu(silu(torch.tensor(X, dtype=torch.float64) @ W1.T + b1) @ W2.T + b2) @ W3.T + b3) @ Wo + bo
    # hi/lo BF16 activations carry 16 significant bits: FP32-level agreement
    np.testing.assert_allclose(got, y.numpy(), rtol=0, atol=2e-5 * float(np.abs(y.numpy()).max()))


@pytest.mark.parametrize("process", [1, 2])
def test_training_data_from_the_plain_kernel(cuda_device, process):
    K, q, e = training_pairs(process, 20000)
    s = Surrogate(process)
    Xraw, R, valid, _ = s.prepare(K, q, e)
    Xraw, R, valid = Xraw.cpu().numpy(), R.cpu().numpy(), valid.cpu().numpy()
    for i, z in enumerate(BATCH_Z):
        m = e == i
        d = oracle.dcs(process, K[m], q[m], ELEMENTS[z], MUON_MASS)
        assert np.array_equal(valid[m], d > 0)
    np.testing.assert_allclose(Xraw[:, 0], np.log(K), rtol=1e-6)
    np.testing.assert_allclose(Xraw[:, 1], np.log(q / (K + MUON_MASS)), rtol=1e-6, atol=1e-6)
    assert np.all(np.isfinite(R[valid]))


def test_short_training_reduces_loss_and_checkpoint_roundtrip(cuda_device, tmp_path):
    K, q, e = training_pairs(1, 200_000)
    s = Surrogate(1, batch=2048)
    Xraw, R, valid, _ = s.prepare(K, q, e)
    Xraw, R = Xraw[valid], R[valid]
    s.fit_norm(Xraw, R)
    s.set_params(init_params(0), s.norm)
    X, T = s.normalise(Xraw, R)
    losses = s.fit(X, T, steps=400, lr=2e-3, lr_final=1e-4).cpu().numpy()
    assert losses[-20:].mean() < 0.05 * losses[0]
    path = tmp_path / "surrogate.npz"
    s.save(path)
    s2 = Surrogate.load(path, batch=2048)
    a, b = s.predict(X[:5000]), s2.predict(X[:5000])
    assert torch.equal(a, b)
    p1, m1, v1, st1 = s.get_params()
    p2, m2, v2, st2 = s2.get_params()
    assert st1 == st2 == 400 and np.array_equal(p1, p2) and np.array_equal(m1, m2)


def test_recipe_with_a_stage_two_smaller_than_a_batch(cuda_device):
    """A very short first stage can leave fewer kept samples than one batch;
    the recipe then skips stage 2 (and says so) instead of failing."""
    from noa_gb300.surrogate import train_recipe
    s = train_recipe(1, n_valid=200_000, steps1=20, steps2=20, batch=8192, heldout=100_000)
    assert s.info["steps"] in (20, 40)
    assert (s.info["stage2_pairs"] == 0) == (s.info["steps"] == 20)
    assert s.trust is not None
    s.close()
