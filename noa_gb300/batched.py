"""Batched multi-element DCS: one persistent launch for many elements.

Python side of the noa_dcs_batch_plan_* C ABI (include/noa_dcs.h).  A
BatchPlan evaluates one process for up to 16 segments (element, count) whose
pairs lie back to back in K, q and result.  `autotune` times the engine's
tile shapes on a prefix of the data and remembers the winner in a JSON cache
(keyed by GPU, process, precision and size), `execute_graph` replays the work
as one CUDA graph.  No counterpart in the reference, which evaluates one
element per call.
"""
import ctypes
import json
import math
import os

import torch

from . import _lib
from .elements import MUON_MASS

DEFAULT_CACHE = os.path.join(os.path.expanduser("~"), ".cache", "noa_gb300", "autotune.json")


def _check(status):
    if status != _lib.SUCCESS:
        raise _lib.DcsError(status, _lib.load().noa_dcs_batch_last_error().decode())


class BatchPlan:
    def __init__(self, process, elements, counts, mass=MUON_MASS, precision="fp64", tolerance=None):
        lib = _lib.load()
        self.process = process if isinstance(process, int) else _lib.PROCESSES.index(process)
        self.precision = precision
        self.counts = [int(c) for c in counts]
        self.n = sum(self.counts)
        n_seg = len(self.counts)
        els = (_lib.Element * max(1, n_seg))(*[_lib.element_struct(e) for e in elements])
        cnt = (ctypes.c_int64 * max(1, n_seg))(*self.counts)
        handle = ctypes.c_void_p()
        _check(lib.noa_dcs_batch_plan_create(ctypes.byref(handle), self.process, _lib.PRECISIONS[precision], n_seg,
                                             els, cnt, float(mass)))
        self._h = handle
        if tolerance is not None:
            _check(lib.noa_dcs_batch_plan_set_tolerance(self._h, ctypes.c_float(tolerance)))

    def _args(self, result, K, q):
        for t, name in ((result, "result"), (K, "K"), (q, "q")):
            if t.dtype != torch.float64 or not t.is_cuda or not t.is_contiguous() or t.numel() != self.n:
                raise RuntimeError(f"{name} must be a contiguous float64 CUDA tensor of {self.n} elements")
        return result.data_ptr(), K.data_ptr(), q.data_ptr()

    @property
    def tile(self):
        t, i, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _check(_lib.load().noa_dcs_batch_plan_get_tile(self._h, ctypes.byref(t), ctypes.byref(i), ctypes.byref(c)))
        return t.value, i.value, c.value

    def set_tile(self, threads, items, ctas_per_sm):
        _check(_lib.load().noa_dcs_batch_plan_set_tile(self._h, threads, items, ctas_per_sm))

    def _cache_key(self):
        dev = torch.cuda.get_device_name()
        return f"{dev}|{_lib.PROCESSES[self.process]}|{self.precision}|seg{len(self.counts)}|n2^{int(math.log2(max(self.n, 1)))}"

    def autotune(self, result, K, q, sample_per_segment=1 << 20, cache=DEFAULT_CACHE):
        """Picks the fastest tile shape (cached in `cache`, a JSON file; None
        disables the cache) and returns it as (threads, items, ctas_per_sm)."""
        key = self._cache_key()
        table = {}
        if cache and os.path.exists(cache):
            try:
                with open(cache) as f:
                    table = json.load(f)
            except (OSError, ValueError):
                table = {}
        if key in table:
            self.set_tile(*table[key])
            return self.tile
        r, k, qq = self._args(result, K, q)
        stream = torch.cuda.current_stream().cuda_stream
        _check(_lib.load().noa_dcs_batch_plan_autotune(self._h, r, k, qq, stream, int(sample_per_segment)))
        if cache:
            table[key] = list(self.tile)
            os.makedirs(os.path.dirname(cache), exist_ok=True)
            tmp = cache + ".tmp"
            with open(tmp, "w") as f:
                json.dump(table, f, indent=1, sort_keys=True)
            os.replace(tmp, cache)
        return self.tile

    def execute(self, result, K, q):
        r, k, qq = self._args(result, K, q)
        _check(_lib.load().noa_dcs_batch_plan_execute(self._h, r, k, qq, torch.cuda.current_stream().cuda_stream))
        return result

    def execute_graph(self, result, K, q):
        r, k, qq = self._args(result, K, q)
        _check(_lib.load().noa_dcs_batch_plan_execute_graph(self._h, r, k, qq,
                                                             torch.cuda.current_stream().cuda_stream))
        return result

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().noa_dcs_batch_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def batch_inputs(zs, counts, seed=None):
    """Concatenated seeded (K, q) for segments of the given counts: segment s
    uses the workload stream at offset s * 2^32, so segments are independent."""
    import numpy as np

    from .workload import SEED, kinetic_recoil
    Ks, qs = [], []
    for s, c in enumerate(counts):
        K, q = kinetic_recoil(int(c), seed=SEED if seed is None else seed, offset=s << 32)
        Ks.append(K)
        qs.append(q)
    return np.concatenate(Ks) if Ks else np.zeros(0), np.concatenate(qs) if qs else np.zeros(0)
