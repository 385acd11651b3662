"""v2 estimation of every comb candidate (computefourier-1.0-2.0.cc:340-419)
against a restatement on the pipeline's own bucket values, and the
pipelined sparse-output batch entry point.

The restatement takes the device's x_samp (natural order), permutations,
comb residues and estimation windows and recomputes every candidate's value
with the reference's operation sequence in FP64 numpy, then the lower
medians at (L-1)/2.  FP64 plans must match it bit for bit, FP32 plans
within the FP32 tolerance of the parity tests.  The plans use explicit
constants (sfft_make_plan_params), so they also reach loop counts outside
the sorting networks' 8..24, small candidate groups, and shapes the oracle
has no constants for; the reference's own constants are covered by the
oracle parity tests.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP32_L1 = 1e-4


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sfft_gb300 import _lib, build
    build.build()
    return torch, _lib, _lib.load()


def _plan(_lib, L, n, k, prm, prec):
    p = _lib.Params(*prm)
    o = _lib.Options(_lib.SFFT_PREC_FP32 if prec == "fp32" else _lib.SFFT_PREC_FP64, -1, 4)
    plan = L.sfft_make_plan_params(n, k, 1, ctypes.byref(p), ctypes.byref(o))
    assert plan, _lib.last_error()
    f = (ctypes.c_long * 11)()
    assert L.sfft_describe_plan_params(n, k, 1, ctypes.byref(p), f, 11) == 11
    names = ["B_loc", "B_thresh", "B_est", "W_Comb", "Comb_loops", "loops_loc", "loops_thresh",
             "loops_est", "w_loc", "w_est", "x_samp_size"]
    return plan, dict(zip(names, (int(v) for v in f)))


def _fetch(L, plan, what, count, dtype):
    buf = np.empty(count, dtype=dtype)
    c = L.sfft_debug_fetch(plan, what, buf.ctypes.data, count)
    assert c >= 0
    return buf[:c]


def restated_estimates(n, pp, xs, ai, comb, win_loc, win_est):
    """(frequencies, values) of every comb candidate, FP64, in the
    reference's operation order."""
    Ll, L = pp["loops_loc"], pp["loops_loc"] + pp["loops_est"]
    W = pp["W_Comb"]
    f = (np.arange(n // W, dtype=np.int64)[:, None] * W + comb[None, :]).ravel()
    re = np.empty((L, f.size))
    im = np.empty((L, f.size))
    for j in range(L):
        B = pp["B_loc"] if j < Ll else pp["B_est"]
        off = min(j, Ll) * pp["B_loc"] + max(0, j - Ll) * pp["B_est"]
        q = n // B
        win = (win_loc if j < Ll else win_est).reshape(-1, 4)
        p = (f * int(ai[j])) % n
        hashed, dist = p // q, p % q
        up = dist > q // 2
        hashed = np.where(up, (hashed + 1) % B, hashed)
        dist = np.where(up, dist - q, dist)
        m = dist + (q - 1) // 2
        v = xs[off + hashed]
        a, b = v.real, v.imag
        c, d, den = win[m, 0], win[m, 1], win[m, 2]
        re[j] = (a * c + b * d) / den
        im[j] = (a * d - b * c) / den
    loc = (L - 1) // 2
    return f, np.sort(re, axis=0)[loc] + 1j * np.sort(im, axis=0)[loc]


# (n, k, (Bcst_loc, Bcst_est, Comb_cst, loc, est, thresh, comb loops, tol, tol))
CASES = [
    (1 << 22, 100, (1.0, 1.0, 2.0, 3, 3, 2, 1, 1e-8, 1e-8)),      # L = 6: full sort
    (1 << 20, 50, (1.0, 1.0, 2.0, 4, 24, 3, 1, 1e-8, 1e-8)),      # L = 28
    (1 << 18, 40, (2.0, 2.0, 16.0, 4, 12, 3, 2, 1e-8, 1e-8)),     # 64 candidates per comb residue
    (1 << 22, 300, (1.0, 0.5, 2.0, 4, 16, 3, 1, 1e-8, 1e-8)),     # different loc / est bucket counts
]


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("n,k,prm", CASES)
def test_estimation_matches_restatement(env, n, k, prm, prec):
    torch, _lib, L = env
    from sfft_gb300 import signals
    plan, pp = _plan(_lib, L, n, k, prm, "fp64")
    Lr = pp["loops_loc"] + pp["loops_est"]
    W, ql, qe = pp["W_Comb"], n // pp["B_loc"], n // pp["B_est"]
    x, _, _ = signals.make_signal(n, k, 17, snr_db=30.0)
    xd = torch.from_numpy(x).cuda()
    cap = L.sfft_output_capacity(plan)

    def run(pl, dt):
        idx = torch.empty(cap, dtype=torch.int32, device="cuda")
        val = torch.empty(cap, dtype=dt, device="cuda")
        cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
        ptr = (ctypes.c_void_p * 1)(xd.data_ptr())
        seeds = (ctypes.c_uint * 1)(23)
        assert L.sfft_exec_batch_ex(pl, 1, ptr, _lib.SFFT_IN_C128, seeds, ctypes.c_void_p(idx.data_ptr()),
                                    ctypes.c_void_p(val.data_ptr()), ctypes.c_void_p(cnt.data_ptr()), cap,
                                    None) == 0, _lib.last_error()
        assert L.sfft_sync(pl) == 0, _lib.last_error()
        c = int(cnt[0])
        gi = idx[:c].cpu().numpy()
        gv = val[:c].cpu().numpy().astype(np.complex128)
        o = np.argsort(gi)
        return gi[o], gv[o]

    # FP64 windows (c, d, c^2 + d^2): the same filters for both precisions
    wl = _fetch(L, plan, 8, 4 * ql, np.float64)
    we = _fetch(L, plan, 9, 4 * qe, np.float64)
    pl = plan if prec == "fp64" else _plan(_lib, L, n, k, prm, "fp32")[0]
    gi, gv = run(pl, torch.complex128 if prec == "fp64" else torch.complex64)
    xs = _fetch(L, pl, 3, pp["x_samp_size"], np.complex128 if prec == "fp64" else np.complex64)
    perm = _fetch(L, pl, 0, 2 * Lr, np.int32)
    comb = _fetch(L, pl, 4, W, np.int32).astype(np.int64)
    rf, rv = restated_estimates(n, pp, xs.astype(np.complex128), perm[Lr:], comb, wl, we)
    o = np.argsort(rf)
    rf, rv = rf[o], rv[o]
    np.testing.assert_array_equal(gi, rf)          # every candidate of the device's comb residues
    if prec == "fp64":
        np.testing.assert_array_equal(gv, rv)
    else:
        # FP32 windows and arithmetic against FP64 arithmetic on the same
        # FP32 bucket values
        l1 = np.abs(gv.real - rv.real) + np.abs(gv.imag - rv.imag)
        assert float(np.max(l1)) <= FP32_L1, float(np.max(l1))
        L.sfft_free_plan(pl)
    L.sfft_free_plan(plan)


def test_exec_many_sparse_matches_sequential_oracle(env, oracle_lib):
    """sfft_exec_many_sparse on page-locked host buffers: the pipelined
    chunks must give each signal the oracle's result under the same
    sequential draws (as sfft_exec_many does)."""
    torch, _lib, L = env
    from sfft_gb300 import signals
    from sfft_gb300.sfft import sfft
    n, k, num = 1 << 16, 50, 7
    for v in (1, 2):
        xs = [signals.make_signal(n, k, 40 + s, snr_db=40.0)[0] for s in range(num)]
        op = oracle_lib.OraclePlan(n, k, v - 1)
        oracle_lib.seed_libc(91)
        refs = [op.exec(x) for x in xs]
        p = sfft(n, k, v, max_batch=2)              # one signal per chunk: seven pipelined chunks
        cap = p.capacity
        nb = n * 16
        hin = [L.sfft_malloc(nb) for _ in range(num)]
        for h, x in zip(hin, xs):
            ctypes.memmove(h, x.ctypes.data, nb)
        hidx = L.sfft_malloc(4 * cap * num)
        hval = L.sfft_malloc(16 * cap * num)
        hcnt = np.zeros(num, dtype=np.int32)
        pin = (ctypes.c_void_p * num)(*hin)
        oracle_lib.seed_libc(91)
        rc = L.sfft_exec_many_sparse(p.sfft_plan, num, pin, ctypes.c_void_p(hidx), ctypes.c_void_p(hval),
                                     ctypes.c_void_p(hcnt.ctypes.data), cap)
        assert rc == 0, _lib.last_error()
        idx = np.ctypeslib.as_array((ctypes.c_int * (cap * num)).from_address(hidx)).reshape(num, cap)
        val = np.ctypeslib.as_array((ctypes.c_double * (2 * cap * num)).from_address(hval)).view(
            np.complex128).reshape(num, cap)
        for s in range(num):
            c = int(hcnt[s])
            o = np.argsort(idx[s, :c])
            np.testing.assert_array_equal(idx[s, :c][o], refs[s][0])
            np.testing.assert_array_equal(val[s, :c][o], refs[s][1])
        for h in hin + [hidx, hval]:
            L.sfft_free(h)
