"""ctypes view of the CPU oracle (liboracle.so) and of the reference build.

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and
bench.py's CPU legs, always as the checker.  The product never imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")

_lib = None
_libc = ctypes.CDLL("libc.so.6")
_libc.srandom.argtypes = [ctypes.c_uint]
_libc.srand48.argtypes = [ctypes.c_long]


def build(quiet=True):
    """Compile liboracle.so (gcc, -ffp-contract=off)."""
    cmd = ["make", "-C", HERE]
    if quiet:
        cmd.append("-s")
    subprocess.check_call(cmd)


def build_ref():
    """Compile the unmodified reference against the shim (needs its sources)."""
    subprocess.check_call(["make", "-C", HERE, "-s", "ref"])


def seed_libc(seed):
    """Seed glibc random() and drand48(), the reference's RNG streams."""
    _libc.srandom(int(seed) & 0xFFFFFFFF)
    _libc.srand48(int(seed))


class Params(ctypes.Structure):
    _fields_ = [(f, ctypes.c_int) for f in (
        "version", "n", "k", "B_loc", "B_thresh", "B_est", "W_Comb", "Comb_loops",
        "loops_loc", "loops_thresh", "loops_est", "w_loc", "w_est")] + [
        ("x_samp_size", ctypes.c_long)] + [(f, ctypes.c_int) for f in (
            "B_g1", "w_g1", "B_g2", "w_g2", "W_Man", "Gauss_loops", "Gauss2_loops",
            "Man_loops")]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        vp, ip, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)
        L.oracle_make_plan.restype = vp
        L.oracle_make_plan.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.oracle_get_params.argtypes = [vp, ctypes.POINTER(Params)]
        L.oracle_filter_time.restype = dp
        L.oracle_filter_time.argtypes = [vp, ctypes.c_int]
        L.oracle_filter_freq.restype = dp
        L.oracle_filter_freq.argtypes = [vp, ctypes.c_int]
        L.oracle_free_plan.argtypes = [vp]
        L.oracle_exec.restype = ctypes.c_long
        L.oracle_exec.argtypes = [vp, vp, vp, vp, ctypes.c_long]
        L.oracle_exec_many_dense.argtypes = [vp, ctypes.c_int, vp, vp]
        L.oracle_dbg_perm.restype = ip
        L.oracle_dbg_perm.argtypes = [vp, ctypes.c_int]
        L.oracle_dbg_J.restype = ip
        L.oracle_dbg_J.argtypes = [vp]
        L.oracle_dbg_score.restype = ip
        L.oracle_dbg_score.argtypes = [vp]
        L.oracle_dbg_hits.restype = ip
        L.oracle_dbg_hits.argtypes = [vp, ctypes.POINTER(ctypes.c_long)]
        L.oracle_dbg_xsamp.restype = dp
        L.oracle_dbg_xsamp.argtypes = [vp]
        L.oracle_dbg_comb.restype = ip
        L.oracle_dbg_comb.argtypes = [vp, ip]
        L.oracle_dbg_v3.argtypes = [vp, ip]
        L.oracle_dbg_v3_trace.restype = ctypes.c_long
        L.oracle_dbg_v3_trace.argtypes = [vp, vp, ctypes.c_long]
        L.shim_fft.argtypes = [ctypes.c_int, vp, ctypes.c_int]
        _lib = L
    return _lib


def shim_fft(x, sign=-1):
    """The project's reference FFT (fft_shim.c) on a complex128 vector."""
    y = np.ascontiguousarray(x, dtype=np.complex128).copy()
    lib().shim_fft(y.size, y.ctypes.data, int(sign))
    return y


class OraclePlan:
    """One oracle plan: the reference's plan fields, filters and exec."""

    def __init__(self, n, k, version):
        self.lib = lib()
        self.h = self.lib.oracle_make_plan(int(n), int(k), int(version))
        if not self.h:
            raise ValueError(f"oracle: (n={n}, k={k}, v{version + 1}) outside the reference's domain")
        p = Params()
        self.lib.oracle_get_params(self.h, ctypes.byref(p))
        self.params = p.as_dict()
        self.n = p.n

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.oracle_free_plan(self.h)
            self.h = None

    def filter_time(self, which):
        w = self.params["w_loc" if which == 0 else "w_est"] if self.params["version"] < 2 else \
            self.params["w_g1" if which == 0 else "w_g2"]
        ptr = self.lib.oracle_filter_time(self.h, which)
        return np.ctypeslib.as_array(ptr, shape=(2 * w,)).view(np.complex128).copy()

    def filter_freq(self, which):
        ptr = self.lib.oracle_filter_freq(self.h, which)
        return np.ctypeslib.as_array(ptr, shape=(2 * self.n,)).view(np.complex128).copy()

    def exec(self, x, seed=None):
        """Sparse result (sorted frequencies, complex128 values)."""
        x = np.ascontiguousarray(x, dtype=np.complex128)
        assert x.size == self.n
        if seed is not None:
            seed_libc(seed)
        cap = self.n
        idx = np.empty(cap, dtype=np.int32)
        val = np.empty(cap, dtype=np.complex128)
        cnt = self.lib.oracle_exec(self.h, x.ctypes.data, idx.ctypes.data, val.ctypes.data, cap)
        if cnt < 0:
            raise RuntimeError("oracle_exec failed")
        return idx[:cnt].copy(), val[:cnt].copy()

    def exec_many_dense(self, xs):
        outs = [np.empty(self.n, dtype=np.complex128) for _ in xs]
        xs = [np.ascontiguousarray(x, dtype=np.complex128) for x in xs]
        ins = (ctypes.c_void_p * len(xs))(*[x.ctypes.data for x in xs])
        ous = (ctypes.c_void_p * len(xs))(*[o.ctypes.data for o in outs])
        self.lib.oracle_exec_many_dense(self.h, len(xs), ins, ous)
        return outs

    # -- debug views of the last single exec ---------------------------------
    def loops(self):
        return self.params["loops_loc"] + self.params["loops_est"]

    def perm(self):
        L = self.loops()
        a = np.ctypeslib.as_array(self.lib.oracle_dbg_perm(self.h, 0), shape=(L,)).copy()
        ai = np.ctypeslib.as_array(self.lib.oracle_dbg_perm(self.h, 1), shape=(L,)).copy()
        return a, ai

    def J(self):
        L, num = self.loops(), self.params["B_thresh"]
        return np.ctypeslib.as_array(self.lib.oracle_dbg_J(self.h), shape=(L, num)).copy()

    def score(self):
        return np.ctypeslib.as_array(self.lib.oracle_dbg_score(self.h), shape=(self.n,)).copy()

    def hits(self):
        c = ctypes.c_long()
        ptr = self.lib.oracle_dbg_hits(self.h, ctypes.byref(c))
        return np.ctypeslib.as_array(ptr, shape=(max(c.value, 1),))[:c.value].copy()

    def xsamp(self):
        s = self.params["x_samp_size"]
        ptr = self.lib.oracle_dbg_xsamp(self.h)
        return np.ctypeslib.as_array(ptr, shape=(2 * s,)).view(np.complex128).copy()

    def comb(self):
        c = ctypes.c_int()
        ptr = self.lib.oracle_dbg_comb(self.h, ctypes.byref(c))
        return np.ctypeslib.as_array(ptr, shape=(max(c.value, 1),))[:c.value].copy()

    def v3_trace(self):
        buf = np.empty((1 << 16, 5), dtype=np.float64)
        c = self.lib.oracle_dbg_v3_trace(self.h, buf.ctypes.data, buf.shape[0])
        return buf[:c].copy()

    def v3_debug(self):
        v = (ctypes.c_int * 8)()
        self.lib.oracle_dbg_v3(self.h, v)
        keys = ("a", "ai", "b", "init_offset", "init_G_offset", "passes", "early_exit", "found")
        return dict(zip(keys, list(v)))


# ---------------------------------------------------------------------------
# The unmodified reference (oracle/_ref), through its own C API.  Only where
# its sources were present at build time (this is not the case on GPU hosts).

class _Filter(ctypes.Structure):
    _fields_ = [("time", ctypes.c_void_p), ("sizet", ctypes.c_int), ("freq", ctypes.c_void_p)]


class _V12Data(ctypes.Structure):       # src/sfft.h:81-106
    _fields_ = [("threads", ctypes.c_uint), ("fftw_opt", ctypes.c_int),
                ("B_loc", ctypes.c_int), ("B_thresh", ctypes.c_int), ("B_est", ctypes.c_int),
                ("W_Comb", ctypes.c_int), ("Comb_loops", ctypes.c_int),
                ("loops_loc", ctypes.c_int), ("loops_thresh", ctypes.c_int),
                ("loops_est", ctypes.c_int), ("filter", _Filter), ("filter_est", _Filter),
                ("x_samp_size", ctypes.c_size_t), ("loop_sizes", ctypes.c_void_p),
                ("tl", ctypes.c_void_p)]


class _V12TL(ctypes.Structure):         # src/sfft.h:52-79
    _fields_ = [(f, ctypes.c_void_p) for f in (
        "permute", "permuteb", "x_samp", "score", "hits", "Comb_Approved", "J",
        "x_sampt", "samples", "values", "nth_element_storage", "nth_int_element_storage",
        "comb_x_sampt", "comb_samples", "permuted_approved", "p_comb", "p_loc", "p_est")]


class _V3Data(ctypes.Structure):        # src/sfft.h:123-154
    _fields_ = [("threads", ctypes.c_uint)] + [(f, ctypes.c_int) for f in (
        "B_g1", "Gauss_loops", "w_g1", "B_g2", "Gauss2_loops", "w_g2", "W_Man", "Man_loops")] + [
        (f, ctypes.c_void_p) for f in ("filtert1", "filterf1", "filtert2", "filterf2")]


class _Plan(ctypes.Structure):          # src/sfft.h:44-50
    _fields_ = [("version", ctypes.c_int), ("n", ctypes.c_uint), ("k", ctypes.c_uint),
                ("data", ctypes.c_void_p)]


class RefLib:
    """The reference's exported API from oracle/_ref/<name>."""

    def __init__(self, name="libsfft_ref.so"):
        path = os.path.join(REF_DIR, name)
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = ctypes.CDLL(path)
        L.sfft_make_plan.restype = ctypes.POINTER(_Plan)
        L.sfft_make_plan.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.sfft_exec.argtypes = [ctypes.POINTER(_Plan), ctypes.c_void_p, ctypes.c_void_p]
        L.sfft_exec_many.argtypes = [ctypes.POINTER(_Plan), ctypes.c_int, ctypes.c_void_p,
                                     ctypes.c_void_p]
        L.sfft_free_plan.argtypes = [ctypes.POINTER(_Plan)]
        self.L = L

    def plan(self, n, k, version):
        p = self.L.sfft_make_plan(int(n), int(k), int(version), 1 << 6)
        if not p:
            raise ValueError("reference refused the plan")
        return p

    def params(self, plan):
        pl = plan.contents
        if pl.version < 2:
            d = ctypes.cast(pl.data, ctypes.POINTER(_V12Data)).contents
            return dict(B_loc=d.B_loc, B_thresh=d.B_thresh, B_est=d.B_est, W_Comb=d.W_Comb,
                        Comb_loops=d.Comb_loops, loops_loc=d.loops_loc,
                        loops_thresh=d.loops_thresh, loops_est=d.loops_est,
                        w_loc=d.filter.sizet, w_est=d.filter_est.sizet,
                        x_samp_size=d.x_samp_size)
        d = ctypes.cast(pl.data, ctypes.POINTER(_V3Data)).contents
        return dict(B_g1=d.B_g1, w_g1=d.w_g1, B_g2=d.B_g2, w_g2=d.w_g2, W_Man=d.W_Man)

    def filters(self, plan, n):
        pl = plan.contents
        out = []
        if pl.version < 2:
            d = ctypes.cast(pl.data, ctypes.POINTER(_V12Data)).contents
            for f in (d.filter, d.filter_est):
                t = np.ctypeslib.as_array(ctypes.cast(f.time, ctypes.POINTER(ctypes.c_double)),
                                          shape=(2 * f.sizet,)).view(np.complex128).copy()
                fr = np.ctypeslib.as_array(ctypes.cast(f.freq, ctypes.POINTER(ctypes.c_double)),
                                           shape=(2 * n,)).view(np.complex128).copy()
                out.append((t, fr))
        else:
            d = ctypes.cast(pl.data, ctypes.POINTER(_V3Data)).contents
            for tp, fp, w in ((d.filtert1, d.filterf1, d.w_g1), (d.filtert2, d.filterf2, d.w_g2)):
                t = np.ctypeslib.as_array(ctypes.cast(tp, ctypes.POINTER(ctypes.c_double)),
                                          shape=(2 * w,)).view(np.complex128).copy()
                fr = np.ctypeslib.as_array(ctypes.cast(fp, ctypes.POINTER(ctypes.c_double)),
                                           shape=(2 * n,)).view(np.complex128).copy()
                out.append((t, fr))
        return out

    def score(self, plan, n):
        pl = plan.contents
        d = ctypes.cast(pl.data, ctypes.POINTER(_V12Data)).contents
        tl = ctypes.cast(d.tl, ctypes.POINTER(_V12TL)).contents
        return np.ctypeslib.as_array(ctypes.cast(tl.score, ctypes.POINTER(ctypes.c_int)),
                                     shape=(n,)).copy()

    def exec(self, plan, x, seed=None):
        x = np.ascontiguousarray(x, dtype=np.complex128)
        out = np.zeros(x.size, dtype=np.complex128)
        if seed is not None:
            seed_libc(seed)
        self.L.sfft_exec(plan, x.ctypes.data, out.ctypes.data)
        return out

    def free(self, plan):
        self.L.sfft_free_plan(plan)
