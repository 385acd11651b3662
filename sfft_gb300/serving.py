"""Python side of the serving and mixed-batch entry points.

`Server` wraps the continuous-batching server (sfft_server_*): requests of
any (n, k, version, precision) are submitted as they come and waited for in
any order.  `MixedBatch` wraps sfft_mixed_*: signals of different shapes run
as one CUDA graph that later calls replay.  Neither has a counterpart in the
reference binding (python/sfft/sfft.py of sFFT 0.1), which plans one shape
at a time.  Inputs are CUDA tensors (complex128 or complex64) or numpy
arrays (complex128, staged by the library).
"""
import ctypes

import numpy as np

from . import _lib

_PREC = {"fp64": 0, "fp32": 1}


def _signal(x):
    """(pointer, input type, keep-alive) of a CUDA tensor or numpy array."""
    if hasattr(x, "data_ptr") and getattr(x, "is_cuda", False):
        import torch
        if not x.is_contiguous() or x.dtype not in (torch.complex128, torch.complex64):
            raise ValueError("device input must be a contiguous complex128 or complex64 tensor")
        return ctypes.c_void_p(x.data_ptr()), (1 if x.dtype == torch.complex64 else 0), x
    a = np.require(np.asanyarray(x), np.complex128, ["C", "ALIGNED"])
    return ctypes.c_void_p(a.ctypes.data), 0, a


class Server:
    """Continuous-batching server.  tune: 0 the reference's constants, 1
    tuned constants where the reference's are invalid, 2 autotuned constants
    for every v1/v2 request; k_round: 0 none, 1 a quarter-octave grid, 2 powers
    of two (for v3 plans); v2_voted: v2 requests in the voted mode."""

    def __init__(self, device=-1, max_batch=32, hbm_budget_bytes=0, k_round=0, tune=0, v2_voted=False):
        self._L = _lib.load()
        opts = _lib.ServerOptions(int(device), int(max_batch), int(hbm_budget_bytes), int(k_round), int(tune),
                                  1 if v2_voted else 0)
        self._s = self._L.sfft_server_create(ctypes.byref(opts))
        if not self._s:
            raise RuntimeError("sfft_server_create failed: " + _lib.last_error())
        self._keep = {}

    def submit(self, x, k, version=2, precision="fp32", seed=0):
        """Queues one transform of x (length n = len(x)); returns its id."""
        ptr, in_type, keep = _signal(x)
        n = int(keep.numel() if hasattr(keep, "numel") else keep.shape[0])
        rid = self._L.sfft_server_submit(self._s, n, int(k), int(version) - 1, _PREC[precision], ptr, in_type,
                                         int(seed))
        if rid < 0:
            raise RuntimeError("sfft_server_submit failed: " + _lib.last_error())
        self._keep[rid] = (keep, n)
        return rid

    def wait(self, rid, timeout_s=None):
        """(frequencies, coefficients complex128, latency in ms) of a request."""
        tms = -1.0 if timeout_s is None else 1e3 * float(timeout_s)
        cap = self._L.sfft_server_count(self._s, rid, tms)
        if cap == -2:
            raise TimeoutError("request %d not finished" % rid)
        cap = max(int(cap), 1)  # a failed request reports its error below
        idx = np.empty(cap, dtype=np.int32)
        val = np.empty(cap, dtype=np.complex128)
        lat = ctypes.c_double()
        c = self._L.sfft_server_wait_for(self._s, rid, idx.ctypes.data, val.ctypes.data, cap, ctypes.byref(lat), -1.0)
        del self._keep[rid]
        if c < 0:
            raise RuntimeError("request %d failed: %s" % (rid, _lib.last_error()))
        return idx[:c].copy(), val[:c].copy(), lat.value

    def stats(self):
        names = ["batches", "plans_made", "plans_evicted", "deferrals", "plans_cached", "bytes_held", "budget",
                 "queued", "batches_spilled"]
        v = (ctypes.c_long * len(names))()
        m = self._L.sfft_server_stats(self._s, v, len(names))
        return {names[i]: int(v[i]) for i in range(max(0, m))}

    def close(self):
        if getattr(self, "_s", None):
            self._L.sfft_server_destroy(self._s)
            self._s = None
            self._keep.clear()

    def __del__(self):
        self.close()


class MixedBatch:
    """Signals of shapes [(n, k, version, precision), ...] run as one CUDA
    graph per call; tune as in Server (2: autotuned, k rounded to its
    bucket)."""

    def __init__(self, shapes, tune=0, complex64=False, device=-1, persistent=False):
        self._L = _lib.load()
        self.shapes = [(int(n), int(k), int(v), p) for n, k, v, p in shapes]
        num = len(self.shapes)
        if num < 1:
            raise ValueError("no signals")
        arr = lambda vals: (ctypes.c_int * num)(*vals)
        self._m = self._L.sfft_mixed_create(num, arr([s[0] for s in self.shapes]), arr([s[1] for s in self.shapes]),
                                            arr([s[2] - 1 for s in self.shapes]),
                                            arr([_PREC[s[3]] for s in self.shapes]), 1 if complex64 else 0,
                                            int(tune), int(device))
        if not self._m:
            raise RuntimeError("sfft_mixed_create failed: " + _lib.last_error())
        self.plans = int(self._L.sfft_mixed_groups(self._m))
        if persistent and self._L.sfft_mixed_set_persistent(self._m, 1) != 0:
            raise RuntimeError("sfft_mixed_set_persistent failed: " + _lib.last_error())

    def run(self, signals, seeds=None):
        """One execution over device tensors (one per shape), asynchronous."""
        if len(signals) != len(self.shapes):
            raise ValueError("one signal per shape")
        ptrs = []
        for x, (n, _, _, _) in zip(signals, self.shapes):
            ptr, _, keep = _signal(x)
            if not hasattr(keep, "data_ptr") or keep.numel() != n:
                raise ValueError("inputs must be CUDA tensors of their shape's length")
            ptrs.append(ptr.value)
        self._inputs = list(signals)
        ins = (ctypes.c_void_p * len(ptrs))(*ptrs)
        sd = None if seeds is None else (ctypes.c_uint * len(ptrs))(*[int(s) for s in seeds])
        if self._L.sfft_mixed_exec(self._m, ins, sd) != 0:
            raise RuntimeError("sfft_mixed_exec failed: " + _lib.last_error())

    def result(self, s):
        """(frequencies, coefficients complex128) of signal s (waits)."""
        if self._L.sfft_mixed_sync(self._m) != 0:
            raise RuntimeError("sfft_mixed_sync failed: " + _lib.last_error())
        c = int(self._L.sfft_mixed_result_host(self._m, int(s), None, None, 0))
        if c < 0:
            raise RuntimeError(_lib.last_error())
        idx = np.empty(max(c, 1), dtype=np.int32)
        single = self.shapes[s][3] == "fp32" and self.shapes[s][2] < 3
        val = np.empty(max(c, 1), dtype=np.complex64 if single else np.complex128)
        self._L.sfft_mixed_result_host(self._m, int(s), idx.ctypes.data, val.ctypes.data, c)
        return idx[:c].copy(), val[:c].astype(np.complex128)

    def close(self):
        if getattr(self, "_m", None):
            self._L.sfft_mixed_destroy(self._m)
            self._m = None

    def __del__(self):
        self.close()
