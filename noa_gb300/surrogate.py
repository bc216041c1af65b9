"""Learned DCS surrogate: training, held-out trust grid, checkpoints.

Python side of the noa_dcs_mlp_* C ABI.  A Surrogate wraps one network (pair
production or photonuclear) that predicts the residual of log DCS over the
analytic baseline of noa_gb300/csrc/mlp.cuh from (log K, log nu, Z/100,
log A).  Its training data come from the plain FP64 kernels; training runs
on the GPU with the library's BF16 tensor-core forward / backward kernels and
Adam.  A held-out check fills a trust grid over (element, log K, log nu):
cells whose held-out relative DCS error exceeds the bound are answered by the
plain kernels at inference, as is everything outside the trained domain.
No counterpart in the reference.
"""
import ctypes
import math

import numpy as np
import torch

from . import _lib
from .elements import BATCH_Z, ELEMENTS, MUON_MASS

NPARAM = 33793
H = 128
# Trained domain and trust-grid resolution (log K, log nu bins).
LOGK_RANGE = (math.log(1e-3), math.log(1e6))
LOGNU_RANGE = (math.log(1e-7), 0.0)
GRID = (64, 64)


def _check(status):
    if status != _lib.SUCCESS:
        raise _lib.DcsError(status, _lib.load().noa_dcs_mlp_last_error().decode())


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def init_params(seed=0):
    """He-style initialisation for SiLU layers; output layer small."""
    g = np.random.default_rng(seed)
    p = np.zeros(NPARAM, dtype=np.float32)
    o = 0

    def put(shape, scale):
        nonlocal o
        n = int(np.prod(shape))
        p[o:o + n] = (g.standard_normal(n) * scale).astype(np.float32) if scale else 0.0
        o += n

    put((H, 4), math.sqrt(2.0 / 4))
    put((H,), 0)
    put((H, H), math.sqrt(2.0 / H))
    put((H,), 0)
    put((H, H), math.sqrt(2.0 / H))
    put((H,), 0)
    put((H,), math.sqrt(1.0 / H))
    put((1,), 0)
    assert o == NPARAM
    return p


def training_pairs(process, n_valid, elements_z=BATCH_Z, seed=987654, chunk=1 << 22):
    """K, q, element index of about n_valid open pairs (the DCS is non-zero),
    spread evenly over the elements, from the seeded workload law."""
    from .workload import kinetic_recoil
    live = {1: 0.54, 2: 0.20}[process]
    per_el = int(math.ceil(n_valid / len(elements_z) / live * 1.05))
    Ks, qs, es = [], [], []
    for i, z in enumerate(elements_z):
        K, q = kinetic_recoil(per_el, seed=seed + 101 * (i + 1))
        Ks.append(K)
        qs.append(q)
        es.append(np.full(per_el, i, dtype=np.uint8))
    return np.concatenate(Ks), np.concatenate(qs), np.concatenate(es)


class Surrogate:
    def __init__(self, process, batch=4096, elements_z=BATCH_Z, mass=MUON_MASS):
        self.lib = _lib.load()
        self.process = process if isinstance(process, int) else _lib.PROCESSES.index(process)
        self.batch = batch
        self.elements_z = tuple(elements_z)
        self.mass = mass
        h = ctypes.c_void_p()
        _check(self.lib.noa_dcs_mlp_create(ctypes.byref(h), self.process, batch))
        self._h = h
        self.norm = np.zeros(10, dtype=np.float32)
        self.trust = None  # uint8 [n_elements][GRID[0]][GRID[1]]
        self.history = []

    # ------------------------------------------------------------ parameters
    def set_params(self, params, norm, adam_m=None, adam_v=None, step=0):
        self.norm = np.ascontiguousarray(norm, dtype=np.float32)
        params = np.ascontiguousarray(params, dtype=np.float32)
        am = None if adam_m is None else np.ascontiguousarray(adam_m, dtype=np.float32)
        av = None if adam_v is None else np.ascontiguousarray(adam_v, dtype=np.float32)
        _check(self.lib.noa_dcs_mlp_set_params(self._h, params.ctypes.data, am.ctypes.data if am is not None else None,
                                               av.ctypes.data if av is not None else None, int(step),
                                               self.norm.ctypes.data))

    def get_params(self):
        p = np.zeros(NPARAM, dtype=np.float32)
        m = np.zeros(NPARAM, dtype=np.float32)
        v = np.zeros(NPARAM, dtype=np.float32)
        step = ctypes.c_int64()
        _check(self.lib.noa_dcs_mlp_get_params(self._h, p.ctypes.data, m.ctypes.data, v.ctypes.data,
                                               ctypes.byref(step)))
        return p, m, v, step.value

    def state_dict(self):
        p, m, v, step = self.get_params()
        return {"process": self.process, "params": p, "adam_m": m, "adam_v": v, "step": step, "norm": self.norm,
                "elements_z": np.array(self.elements_z), "trust": self.trust if self.trust is not None else
                np.zeros(0, dtype=np.uint8), "mass": self.mass}

    def save(self, path):
        np.savez_compressed(path, **self.state_dict())

    @classmethod
    def load(cls, path, batch=4096):
        z = np.load(path)
        s = cls(int(z["process"]), batch=batch, elements_z=tuple(int(x) for x in z["elements_z"]),
                mass=float(z["mass"]))
        s.set_params(z["params"], z["norm"], z["adam_m"], z["adam_v"], int(z["step"]))
        s.trust = z["trust"] if z["trust"].size else None
        return s

    # ------------------------------------------------------------ data
    def prepare(self, K, q, elem):
        """Raw features, residual targets and validity from the FP64 kernels.
        Returns (Xraw, R, valid, open_zero): valid marks training samples
        (open, DCS > 0); open_zero marks pairs open by the kinematic bounds
        whose DCS is nevertheless 0."""
        dev = torch.device("cuda")
        tK = torch.as_tensor(K, dtype=torch.float64, device=dev)
        tq = torch.as_tensor(q, dtype=torch.float64, device=dev)
        te = torch.as_tensor(elem, dtype=torch.uint8, device=dev)
        n = tK.numel()
        X = torch.empty((n, 4), dtype=torch.float32, device=dev)
        R = torch.empty(n, dtype=torch.float32, device=dev)
        V = torch.empty(n, dtype=torch.uint8, device=dev)
        els = (_lib.Element * len(self.elements_z))(*[_lib.element_struct(ELEMENTS[z]) for z in self.elements_z])
        _check(self.lib.noa_dcs_mlp_prepare(self.process, _ptr(tK), _ptr(tq), _ptr(te), n, els,
                                            len(self.elements_z), self.mass, _ptr(X), _ptr(R), _ptr(V), _stream()))
        return X, R, V == 1, V == 2

    def fit_norm(self, Xraw, R):
        lo = Xraw.min(0).values.cpu().numpy()
        hi = Xraw.max(0).values.cpu().numpy()
        shift = 0.5 * (lo + hi)
        scale = np.where(hi > lo, 2.0 / np.maximum(hi - lo, 1e-12), 1.0)
        r_mean = float(R.mean())
        r_std = float(R.std())
        self.norm = np.concatenate([shift, scale, [r_mean, 1.0 / max(r_std, 1e-12)]]).astype(np.float32)

    def normalise(self, Xraw, R=None):
        shift = torch.as_tensor(self.norm[:4], device=Xraw.device)
        scale = torch.as_tensor(self.norm[4:8], device=Xraw.device)
        X = ((Xraw - shift) * scale).contiguous()
        if R is None:
            return X
        T = ((R - float(self.norm[8])) * float(self.norm[9])).contiguous()
        return X, T

    def residual(self, y):
        """Normalised network output -> residual of log DCS."""
        return float(self.norm[8]) + y / float(self.norm[9])

    # ------------------------------------------------------------ training
    def fit(self, X, T, steps, lr=2e-3, lr_final=2e-5, seed=0, chunk_steps=2000):
        """Adam on normalised data; the batch order is reshuffled every epoch."""
        n = X.shape[0]
        g = torch.Generator(device="cuda").manual_seed(seed)
        losses = torch.empty(steps, dtype=torch.float32, device="cuda")
        done = 0
        epoch_batches = n // self.batch
        # one cosine schedule over all steps, issued in chunks of whole epochs
        while done < steps:
            perm = torch.randperm(n, generator=g, device="cuda").to(torch.int32)
            todo = min(epoch_batches, steps - done, chunk_steps)
            a = lr_final + 0.5 * (lr - lr_final) * (1 + math.cos(math.pi * done / steps))
            b = lr_final + 0.5 * (lr - lr_final) * (1 + math.cos(math.pi * (done + todo) / steps))
            _check(self.lib.noa_dcs_mlp_train(self._h, _ptr(X), _ptr(T), n, _ptr(perm), todo, ctypes.c_float(a),
                                              ctypes.c_float(b), ctypes.c_void_p(losses[done:].data_ptr()),
                                              _stream()))
            done += todo
        torch.cuda.synchronize()
        self.history.append(losses.cpu().numpy())
        return losses

    def predict(self, X):
        out = torch.empty(X.shape[0], dtype=torch.float32, device="cuda")
        _check(self.lib.noa_dcs_mlp_predict(self._h, _ptr(X.contiguous()), _ptr(out), X.shape[0], _stream()))
        return out

    def gradient(self, X, T):
        g = torch.empty(NPARAM, dtype=torch.float32, device="cuda")
        loss = torch.empty(1, dtype=torch.float32, device="cuda")
        _check(self.lib.noa_dcs_mlp_gradient(self._h, _ptr(X.contiguous()), _ptr(T.contiguous()), X.shape[0],
                                             _ptr(g), _ptr(loss), _stream()))
        torch.cuda.synchronize()
        return g, float(loss)

    # ------------------------------------------------------------ trust grid
    def cells(self, Xraw, elem):
        """Trust-grid cell of each sample (raw features), -1 outside the
        trained domain: floor((log - lo) * scale) per axis in float32 with lo
        and scale rounded to float32, the arithmetic of the inference kernel."""
        lk, ln = Xraw[:, 0].float(), Xraw[:, 1].float()
        k_lo, k_sc = float(np.float32(LOGK_RANGE[0])), float(np.float32(GRID[0] / (LOGK_RANGE[1] - LOGK_RANGE[0])))
        n_lo, n_sc = float(np.float32(LOGNU_RANGE[0])), float(np.float32(GRID[1] / (LOGNU_RANGE[1] - LOGNU_RANGE[0])))
        ik = ((lk - k_lo) * k_sc).floor().long()
        inu = ((ln - n_lo) * n_sc).floor().long()
        inside = (ik >= 0) & (ik < GRID[0]) & (inu >= 0) & (inu < GRID[1])
        c = (elem.long() * GRID[0] + ik.clamp(0, GRID[0] - 1)) * GRID[1] + inu.clamp(0, GRID[1] - 1)
        return torch.where(inside, c, torch.full_like(c, -1))

    def lattice(self, points=7):
        """A points x points lattice of (K, q) spanning every trust-grid cell
        of every element, its edges and corners included: returns (K, q,
        element index, cell index) as numpy arrays."""
        gk, gn = GRID
        dk = (LOGK_RANGE[1] - LOGK_RANGE[0]) / gk
        dn = (LOGNU_RANGE[1] - LOGNU_RANGE[0]) / gn
        t = np.linspace(0.0, 1.0, points)
        ik, inu, a, b = np.meshgrid(np.arange(gk), np.arange(gn), t, t, indexing="ij")
        lk = (LOGK_RANGE[0] + (ik + a) * dk).ravel()
        ln = (LOGNU_RANGE[0] + (inu + b) * dn).ravel()
        cell2 = (ik * gn + inu).ravel()
        n_el = len(self.elements_z)
        K = np.tile(np.exp(lk), n_el)
        q = np.tile(np.exp(ln), n_el) * (K + self.mass)   # nu = q / (K + m), as the features
        elem = np.repeat(np.arange(n_el, dtype=np.uint8), lk.size)
        cell = elem.astype(np.int64) * (gk * gn) + np.tile(cell2, n_el)
        return K, q, elem, cell

    def build_trust(self, Xraw, R, valid, elem, bound=1e-3, safety=0.35, open_zero=None, lattice_points=7):
        """Trust grid.  A cell is trusted when (1) every point of a
        lattice_points x lattice_points lattice spanning it, edges and corners
        included, is open with a non-zero DCS and has |predicted - true|
        log DCS (the relative DCS error to first order) at most safety *
        bound, and (2) so do all of its samples in the random held-out set
        (Xraw, R, valid, elem: features, residuals and validity from
        prepare()), none of which may be open with DCS = 0 (open_zero).  The
        lattice takes every cell that touches a kinematic edge (DCS -> 0, where
        log DCS is steep) out, and bounds the error of a smooth network between
        its points; the random samples cover the cell's interior at other
        positions.  The true maximum inside a cell is still only estimated,
        hence the safety factor."""
        ncell = len(self.elements_z) * GRID[0] * GRID[1]
        lim = safety * bound
        # (1) the lattice
        Kl, ql, el, cl = self.lattice(lattice_points)
        Xl, Rl, vl, _ = self.prepare(Kl, ql, el)
        cl = torch.as_tensor(cl, device="cuda")
        ok = torch.zeros(Kl.size, dtype=torch.bool, device="cuda")
        if bool(vl.any()):
            Xn = self.normalise(Xl[vl])
            errl = (self.residual(self.predict(Xn)) - Rl[vl]).abs()
            ok[vl] = errl <= lim
        bad = torch.zeros(ncell, dtype=torch.int64, device="cuda")
        bad.scatter_add_(0, cl, (~ok).long())
        trust = bad == 0
        lattice_trusted = int(trust.sum())
        # (2) the random held-out set
        Xv, Rv, ev = Xraw[valid], R[valid], elem[valid]
        X, _ = self.normalise(Xv, Rv)
        err = (self.residual(self.predict(X)) - Rv).abs()
        cell = self.cells(Xv, ev)
        keep = cell >= 0
        worst = torch.zeros(ncell, dtype=torch.float32, device="cuda")
        worst.scatter_reduce_(0, cell[keep], err[keep], reduce="amax")
        trust &= worst <= lim
        if open_zero is not None and bool(open_zero.any()):
            zc = self.cells(Xraw[open_zero], elem[open_zero])
            zc = zc[zc >= 0]
            trust[zc] = False
        self.trust = trust.to(torch.uint8).cpu().numpy().reshape(len(self.elements_z), *GRID)
        return {"cells_trusted": int(trust.sum()), "cells_lattice_ok": lattice_trusted,
                "heldout_err_max": float(err.max()), "heldout_err_median": float(err.median()),
                "heldout_frac_trusted": float(trust[cell[keep]].float().mean())}

    # ------------------------------------------------------------ inference
    def infer(self, K, q, counts, tolerance=1e-6, trust=None, out=None):
        """DCS of the pairs (K, q) (CUDA float64, segments of `counts` pairs,
        element i = elements_z[i]) through noa_dcs_mlp_infer: the network
        (tcgen05) in trusted cells, the FP32C kernel elsewhere.  Writes into
        `out` when given (CUDA float64, K's size).  Returns (result,
        {"network": n1, "fallback": n2, "status": st})."""
        trust = self.trust if trust is None else trust
        if trust is None:
            raise RuntimeError("no trust grid: call build_trust first")
        tg = self._device_trust(trust)
        if out is None:
            out = torch.empty_like(K)
        elif out.dtype != torch.float64 or not out.is_cuda or not out.is_contiguous() or out.numel() != K.numel():
            raise RuntimeError("out must be a contiguous CUDA float64 tensor of K's size")
        n_seg = len(counts)
        els = (_lib.Element * n_seg)(*[_lib.element_struct(ELEMENTS[z]) for z in self.elements_z[:n_seg]])
        cnt = (ctypes.c_int64 * n_seg)(*[int(c) for c in counts])
        stats = (ctypes.c_ulonglong * 3)()
        lib = self.lib
        st = lib.noa_dcs_mlp_infer(self._h, _ptr(tg), n_seg, els, cnt, self.mass, _ptr(out), _ptr(K), _ptr(q),
                                   ctypes.c_float(tolerance), ctypes.cast(stats, ctypes.c_void_p), _stream())
        if st != _lib.SUCCESS:
            raise _lib.DcsError(st, lib.noa_dcs_mlp_infer_last_error().decode())
        torch.cuda.synchronize()
        return out, {"network": int(stats[0]), "fallback": int(stats[1]), "status": int(stats[2])}

    def _device_trust(self, trust):
        """The trust grid on the GPU, uploaded again only when it changes."""
        host = np.ascontiguousarray(trust, dtype=np.uint8)
        cached = getattr(self, "_trust_dev", None)
        if cached is not None and cached[0].shape == host.shape and np.array_equal(cached[0], host):
            return cached[1]
        tg = torch.as_tensor(host, device="cuda")
        self._trust_dev = (host.copy(), tg)
        return tg

    def close(self):
        if getattr(self, "_h", None):
            self.lib.noa_dcs_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def train_recipe(process, n_valid=10_000_000, steps1=60_000, steps2=150_000, batch=8192, keep_err=2e-2,
                 heldout=2_000_000, bound=1e-3, seed=0, log=None):
    """The surrogate's training recipe: train on all open pairs, drop the
    trust-grid cells whose held-out error exceeds keep_err (they will be
    answered by the plain kernels anyway), train on the rest with a lower
    learning rate, and build the trust grid at `bound` from a held-out set."""
    import time
    t0 = time.time()
    K, q, e = training_pairs(process, n_valid)
    s = Surrogate(process, batch=batch)
    Xraw, R, valid, _ = s.prepare(K, q, e)
    et = torch.as_tensor(e, device="cuda")
    Xv, Rv, ev = Xraw[valid], R[valid], et[valid]
    s.fit_norm(Xv, Rv)
    s.set_params(init_params(seed), s.norm)
    X, T = s.normalise(Xv, Rv)
    s.fit(X, T, steps=steps1, lr=2e-3, lr_final=2e-5, seed=seed)
    Kh, qh, eh = training_pairs(process, heldout, seed=12345)
    Xh, Rh, vh, zh = s.prepare(Kh, qh, eh)
    eht = torch.as_tensor(eh, device="cuda")
    Xn, _ = s.normalise(Xh[vh], Rh[vh])
    err = (s.residual(s.predict(Xn)) - Rh[vh]).abs()
    cell = s.cells(Xh[vh], eht[vh])
    worst = torch.zeros(len(s.elements_z) * GRID[0] * GRID[1], device="cuda")
    k = cell >= 0
    worst.scatter_reduce_(0, cell[k], err[k], reduce="amax")
    tc = s.cells(Xv, ev)
    keep = (tc >= 0) & (worst[tc.clamp(min=0)] <= keep_err)
    # stage 2 needs at least one batch of kept samples (a very short stage 1
    # can leave fewer); without them the model stays as stage 1 left it
    if int(keep.sum()) >= s.batch:
        s.fit(X[keep].contiguous(), T[keep].contiguous(), steps=steps2, lr=5e-4, lr_final=5e-6, seed=seed + 1)
    else:
        steps2 = 0
    info = s.build_trust(Xh, Rh, vh, eht, bound=bound, open_zero=zh)
    info.update({"train_seconds": time.time() - t0, "training_pairs": int(Xv.shape[0]),
                 "stage2_pairs": int(keep.sum()) if steps2 else 0, "steps": steps1 + steps2, "batch": batch})
    if log:
        log(info)
    s.info = info
    return s


def _main(argv=None):
    """Command line: train and save a surrogate, or evaluate a saved one.

        python -m noa_gb300.surrogate train PROCESS OUT.npz [--pairs N] [--steps1 S] [--steps2 S]
        python -m noa_gb300.surrogate infer MODEL.npz [--queries N] [--repeat R]
                                         [--trust model|all|none] [--fp32c]

    infer evaluates N seeded queries over the model's elements (equal
    counts); --trust all sends every open pair to the network and none sends
    none (the pipeline without the network), model uses the trained trust
    grid; --fp32c also times the FP32C batched engine on the same queries.
    Times are CUDA-event milliseconds of one call (the last of R)."""
    import argparse
    import json

    from .batched import BatchPlan, batch_inputs
    ap = argparse.ArgumentParser(prog="python -m noa_gb300.surrogate")
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("process", type=int, choices=[1, 2])
    t.add_argument("out")
    t.add_argument("--pairs", type=float, default=1e7)
    t.add_argument("--steps1", type=int, default=60_000)
    t.add_argument("--steps2", type=int, default=150_000)
    i = sub.add_parser("infer")
    i.add_argument("model")
    i.add_argument("--queries", type=float, default=1e7)
    i.add_argument("--repeat", type=int, default=3)
    i.add_argument("--trust", choices=["model", "all", "none"], default="model")
    i.add_argument("--fp32c", action="store_true")
    a = ap.parse_args(argv)
    if a.cmd == "train":
        s = train_recipe(a.process, n_valid=int(a.pairs), steps1=a.steps1, steps2=a.steps2)
        s.save(a.out)
        print(json.dumps(s.info))
        return
    s = Surrogate.load(a.model)
    nq = int(a.queries)
    counts = [nq // len(s.elements_z)] * len(s.elements_z)
    counts[-1] += nq - sum(counts)
    K, q = batch_inputs(s.elements_z, counts, seed=777)
    tk, tq = torch.from_numpy(K).cuda(), torch.from_numpy(q).cuda()
    del K, q
    out = torch.empty_like(tk)
    shape = (len(s.elements_z), *GRID)
    trust = {"model": None, "all": np.ones(shape, np.uint8), "none": np.zeros(shape, np.uint8)}[a.trust]

    def timed(fn):
        ms, res = 0.0, None
        for _ in range(max(1, a.repeat)):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            res = fn()
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
        return ms, res

    ms, (_, st) = timed(lambda: s.infer(tk, tq, counts, trust=trust, out=out))
    line = {"queries": nq, "trust": a.trust, "ms": ms, "evals_per_s": nq / (ms * 1e-3), **st}
    if a.fp32c:
        with BatchPlan(s.process, [ELEMENTS[z] for z in s.elements_z], counts, s.mass, "fp32c") as plan:
            plan.set_tile(256, 8, 2)
            line["fp32c_engine_ms"], _ = timed(lambda: plan.execute(out, tk, tq))
    print(json.dumps(line))


if __name__ == "__main__":
    _main()
