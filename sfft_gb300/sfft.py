"""Python interface of the GB300 sparse FFT engine.

`sfft` keeps the class, constructor arguments and `execute` semantics of the
reference binding (python/sfft/sfft.py:33-85 of sFFT 0.1): a plan for
(length, sparsity, version) and a dense complex128 result.  Differences:
Python 3 / numpy 2; the (n, k) whitelist of v1/v2 (:10-31) is a warning,
not an error, because the library validates the domain itself; errors
raise with the library's message; and `execute_sparse`, `precision`,
`voted`, device-array input and batched execution are added.
"""
import ctypes
import warnings

import numpy as np

from . import _lib
from ._lib import FFTW_ESTIMATE, FFTW_MEASURE  # noqa: F401  (values of fftw3.h)

V1_V2_INPUT_PARAMETERS = (
    [{"size": 1 << e, "sparsity": 50} for e in range(13, 25)]
    + [{"size": 4194304, "sparsity": s} for s in (100, 200, 500, 1000, 2000, 2500, 4000)]
)


def _as_int(name, v):
    if not isinstance(v, (int, np.integer)):
        raise TypeError(f"{name} is not an integer")
    return int(v)


class sfft:
    """A sparse FFT plan (python/sfft/sfft.py:33-85)."""

    def __init__(self, length=16384, sparsity=50, version=1, optimization=FFTW_ESTIMATE,
                 precision="fp64", device=-1, max_batch=16, voted=False):
        length = _as_int("length", length)
        sparsity = _as_int("sparsity", sparsity)
        version = _as_int("version", version)
        optimization = _as_int("optimization", optimization)
        if version not in (1, 2, 3):
            raise ValueError("sFFT version %d is not valid.  Try 1, 2, or 3." % version)
        if version in (1, 2) and {"size": length, "sparsity": sparsity} not in V1_V2_INPUT_PARAMETERS:
            warnings.warn("n = %d and k = %d is not a tuned parameter combination for sFFT version %d"
                          % (length, sparsity, version))
        if optimization not in (FFTW_MEASURE, FFTW_ESTIMATE):
            raise ValueError("FFTW optimization %d is not valid." % optimization)
        if precision not in ("fp64", "fp32"):
            raise ValueError("precision must be 'fp64' or 'fp32'")
        self.length, self.sparsity, self.version = length, sparsity, version
        self.optimization, self.precision = optimization, precision
        self._L = _lib.load()
        opt = _lib.Options(_lib.SFFT_PREC_FP32 if precision == "fp32" else _lib.SFFT_PREC_FP64,
                           int(device), int(max_batch))
        self.sfft_plan = self._L.sfft_make_plan_ex(length, sparsity, version - 1, FFTW_ESTIMATE,
                                                   ctypes.byref(opt))
        if not self.sfft_plan:
            raise RuntimeError("sfft_make_plan failed: " + _lib.last_error())
        if voted:  # v2 only: estimate the candidates that pass the vote (not the reference's list)
            if version != 2 or self._L.sfft_plan_v2_voted(self.sfft_plan, 1) != 0:
                raise ValueError("the voted mode applies to version 2 plans: " + _lib.last_error())
        self.voted = bool(voted)
        self.capacity = int(self._L.sfft_output_capacity(self.sfft_plan))

    # -- the reference's method ---------------------------------------------
    def execute(self, a):
        """Dense result: an n-point complex128 array (python/sfft/sfft.py:76-82)."""
        a = np.require(np.asanyarray(a), np.complex128, ["C", "ALIGNED"])
        if a.shape != (self.length,):
            raise ValueError(f"input must have shape ({self.length},)")
        b = np.empty_like(a)
        _lib.load().sfft_last_error()
        self._L.sfft_exec(self.sfft_plan, a.ctypes.data, b.ctypes.data)
        err = _lib.last_error()
        if err:
            raise RuntimeError("sfft_exec failed: " + err)
        return b

    # -- additions -------------------------------------------------------------
    def execute_sparse(self, a):
        """(frequencies int32, coefficients complex128) of one transform.

        `a` may be a numpy array or a CUDA tensor (complex128)."""
        ptr, keep = _input_pointer(a, self.length)
        idx = np.empty(self.capacity, dtype=np.int32)
        val = np.empty(self.capacity, dtype=np.complex128)
        c = self._L.sfft_exec_sparse(self.sfft_plan, ptr, idx.ctypes.data, val.ctypes.data, self.capacity)
        del keep
        if c < 0:
            raise RuntimeError("sfft_exec_sparse failed: " + _lib.last_error())
        return idx[:c].copy(), val[:c].copy()

    def execute_many(self, arrays):
        """Dense results of several signals (sfft_exec_many)."""
        ins = [np.require(np.asanyarray(a), np.complex128, ["C", "ALIGNED"]) for a in arrays]
        outs = [np.empty_like(a) for a in ins]
        pin = (ctypes.c_void_p * len(ins))(*[a.ctypes.data for a in ins])
        pout = (ctypes.c_void_p * len(outs))(*[o.ctypes.data for o in outs])
        self._L.sfft_exec_many(self.sfft_plan, len(ins), pin, pout)
        err = _lib.last_error()
        if err:
            raise RuntimeError("sfft_exec_many failed: " + err)
        return outs

    def debug(self, what, count, dtype=np.int32):
        buf = np.empty(count, dtype=dtype)
        c = self._L.sfft_debug_fetch(self.sfft_plan, int(what), buf.ctypes.data, count)
        if c < 0:
            raise RuntimeError("sfft_debug_fetch failed: " + _lib.last_error())
        return buf[:c]

    def __del__(self):
        plan = getattr(self, "sfft_plan", None)
        if plan:
            self._L.sfft_free_plan(plan)
            self.sfft_plan = None


def _input_pointer(a, n):
    """Device pointer of a CUDA tensor, or host pointer of a numpy array."""
    if hasattr(a, "data_ptr") and getattr(a, "is_cuda", False):
        import torch
        if a.dtype != torch.complex128 or a.numel() != n or not a.is_contiguous():
            raise ValueError("device input must be a contiguous complex128 tensor of length n")
        return ctypes.c_void_p(a.data_ptr()), a
    arr = np.require(np.asanyarray(a), np.complex128, ["C", "ALIGNED"])
    if arr.shape != (n,):
        raise ValueError(f"input must have shape ({n},)")
    return ctypes.c_void_p(arr.ctypes.data), arr


def describe_plan(n, k, version):
    """Plan parameters (host-only; the reference's values)."""
    fields = (ctypes.c_long * 11)()
    m = _lib.load().sfft_describe_plan(int(n), int(k), int(version) - 1, fields, 11)
    if m < 0:
        raise ValueError(_lib.last_error())
    names = (["B_loc", "B_thresh", "B_est", "W_Comb", "Comb_loops", "loops_loc", "loops_thresh",
              "loops_est", "w_loc", "w_est", "x_samp_size"] if version < 3
             else ["W_Man", "B_g1", "w_g1", "B_g2", "w_g2"])
    return {nm: int(fields[i]) for i, nm in enumerate(names[:m])}


def describe_filter(n, k, version, which):
    """(time taps, n-point spectrum) of a plan's filter, complex128."""
    L = _lib.load()
    w = L.sfft_describe_filter(int(n), int(k), int(version) - 1, int(which), None, 0, None, 0)
    if w < 0:
        raise ValueError(_lib.last_error())
    t = np.empty(w, dtype=np.complex128)
    f = np.empty(n, dtype=np.complex128)
    r = L.sfft_describe_filter(int(n), int(k), int(version) - 1, int(which), t.ctypes.data, 2 * w,
                               f.ctypes.data, 2 * n)
    if r < 0:
        raise ValueError(_lib.last_error())
    return t, f
