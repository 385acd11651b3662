"""GPU parity: the CUDA path through the C-ABI against the CPU oracle on the
same seeded inputs and the same glibc random()/drand48() stream.

FP64 v1/v2: support, values, permutations, selected buckets, vote counts
and bucket values must be bit-identical.  v3: identical support and values
within 1e-10 relative (its exec calls atan2/sin/cos, whose CUDA and glibc
implementations differ in the last bits, and peels with atomics).
FP32 v1/v2: identical support and per-entry L1 error <= 1e-4 against the
FP64 oracle.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

V3_RTOL = 1e-10
FP32_L1 = 1e-4


@pytest.fixture(scope="module")
def S(oracle_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sfft_gb300 import build
    build.build()
    from sfft_gb300 import sfft as S
    return S


def _sorted(idx, val):
    o = np.argsort(idx, kind="stable")
    return idx[o], val[o]


def _run(S, O, n, k, v, seed, x, prec="fp64"):
    op = O.OraclePlan(n, k, v - 1)
    oi, ov = op.exec(x, seed=seed)
    g = S.sfft(n, k, v, precision=prec)
    O.seed_libc(seed)
    gi, gv = _sorted(*g.execute_sparse(x))
    return op, oi, ov, g, gi, gv


V12_CASES = [
    # (n, k, version, seed, magnitudes, snr_db)
    (1 << 16, 50, 1, 0, None, None),            # C1 shape
    (1 << 16, 50, 1, 5, None, None),
    (8192, 50, 1, 3, None, None),
    (1 << 16, 50, 2, 0, None, None),
    (1 << 16, 50, 2, 2, None, 40.0),
    (1 << 20, 50, 2, 4, None, None),
    (1 << 22, 100, 1, 11, None, None),
    (1 << 22, 100, 2, 7, (0.1, 10.0), 20.0),    # C4 shape (metric workload)
    (1 << 24, 50, 1, 13, None, None),           # B_loc = 16384: global-memory FFTs
    (256, 2, 1, 9, None, None),                 # smallest tuned-free domain
    (256, 2, 2, 9, None, None),
]


@pytest.mark.parametrize("n,k,v,seed,mag,snr", V12_CASES)
def test_v12_fp64_bit_exact(S, oracle_lib, n, k, v, seed, mag, snr):
    from sfft_gb300 import signals
    x, _, _ = signals.make_signal(n, k, seed, mag=mag, snr_db=snr)
    op, oi, ov, g, gi, gv = _run(S, oracle_lib, n, k, v, seed, x)
    np.testing.assert_array_equal(gi, oi)
    np.testing.assert_array_equal(gv, ov)
    L = op.loops()
    perm = g.debug(0, 2 * L)
    a, ai = op.perm()
    np.testing.assert_array_equal(perm[:L], a)
    np.testing.assert_array_equal(perm[L:], ai)
    np.testing.assert_array_equal(g.debug(1, L * op.params["B_thresh"]).reshape(L, -1), op.J())
    np.testing.assert_array_equal(g.debug(2, n), op.score())
    xs = g.debug(3, op.params["x_samp_size"], np.complex128)
    np.testing.assert_array_equal(xs, op.xsamp())
    if v == 2:
        np.testing.assert_array_equal(g.debug(4, n), op.comb())


@pytest.mark.parametrize("v,prec", [(1, "fp64"), (2, "fp64"), (1, "fp32"), (2, "fp32")])
def test_v12_global_memory_fft_path(S, oracle_lib, monkeypatch, v, prec):
    """Bucket and comb FFTs forced through the multi-launch global-memory
    Stockham path (as plans with more than 8192 / 16384 buckets use)."""
    from sfft_gb300 import signals
    monkeypatch.setenv("SFFT_GB300_MAX_SMEM_FFT", "256")
    n, k, seed = 1 << 16, 50, 3
    x, pos, vals = signals.make_signal(n, k, seed, snr_db=40.0)
    op, oi, ov, g, gi, gv = _run(S, oracle_lib, n, k, v, seed, x, prec=prec)
    if prec == "fp64":
        np.testing.assert_array_equal(gi, oi)
        np.testing.assert_array_equal(gv, ov)
        L = op.loops()
        np.testing.assert_array_equal(g.debug(2, n), op.score())
        np.testing.assert_array_equal(g.debug(1, L * op.params["B_thresh"]).reshape(L, -1), op.J())
    else:
        tau = 0.5 * float(np.min(np.abs(vals)))
        np.testing.assert_array_equal(gi[np.abs(gv) >= tau], oi[np.abs(ov) >= tau])


@pytest.mark.parametrize("v", [1, 2])
def test_v12_zero_signal_ties(S, oracle_lib, v):
    """All buckets equal: the selection takes the first 2k indices."""
    n, k = 1 << 14, 20
    x = np.zeros(n, dtype=np.complex128)
    op, oi, ov, g, gi, gv = _run(S, oracle_lib, n, k, v, 123, x)
    np.testing.assert_array_equal(gi, oi)
    np.testing.assert_array_equal(gv, ov)
    L = op.loops()
    np.testing.assert_array_equal(g.debug(1, L * 2 * k).reshape(L, -1), op.J())
    np.testing.assert_array_equal(g.debug(2, n), op.score())


V3_CASES = [
    (1 << 16, 50, 1),
    (1 << 18, 100, 1),
    (1 << 18, 100, 2),
    (1 << 20, 200, 3),
    (1 << 24, 1000, 1),    # C2 shape
    (1 << 20, 500, 4),     # comb width 4096
    (1 << 20, 1700, 5),    # comb width 16384: Mansour FFTs in global memory
]


@pytest.mark.parametrize("n,k,seed", V3_CASES)
def test_v3_support_and_values(S, oracle_lib, n, k, seed):
    from sfft_gb300 import signals
    x, _, _ = signals.make_signal(n, k, seed)
    op, oi, ov, g, gi, gv = _run(S, oracle_lib, n, k, 3, seed, x)
    np.testing.assert_array_equal(gi, oi)
    scale = max(1.0, float(np.max(np.abs(ov))))
    assert float(np.max(np.abs(gv - ov))) <= V3_RTOL * scale
    d = g.debug(0, 5)
    dbg = op.v3_debug()
    assert list(d) == [dbg["a"], dbg["ai"], dbg["b"], dbg["init_offset"], dbg["init_G_offset"]]


def test_v3_early_return_is_empty(S, oracle_lib):
    """The reference returns before writing out[] when the comb stage finds
    all k tones (src/computefourier-3.0.cc:859-860)."""
    from sfft_gb300 import signals
    n, k, seed = 1 << 14, 8, 21
    x, _, _ = signals.make_signal(n, k, seed)
    op, oi, ov, g, gi, gv = _run(S, oracle_lib, n, k, 3, seed, x)
    assert oi.size == 0 and gi.size == 0
    assert op.v3_debug()["early_exit"] == 1


FP32_CASES = [
    (1 << 16, 50, 1, 0, None, None),
    (1 << 16, 50, 2, 2, None, 40.0),
    (1 << 22, 100, 2, 7, (0.1, 10.0), 20.0),    # C4: the mixed-precision workload
]


@pytest.mark.parametrize("n,k,v,seed,mag,snr", FP32_CASES)
def test_v12_fp32_support_and_l1(S, oracle_lib, n, k, v, seed, mag, snr):
    """Recovered support {f : |X_f| >= tau}, tau = half the smallest true
    magnitude, must equal the FP64 oracle's; every coefficient both write
    must agree within L1 <= 1e-4.  (The raw written set of v1 can differ in
    entries of size ~1e-8: FP32 rounding reorders noise-floor buckets.)"""
    from sfft_gb300 import signals
    x, pos, vals = signals.make_signal(n, k, seed, mag=mag, snr_db=snr)
    op, oi, ov, g, gi, gv = _run(S, oracle_lib, n, k, v, seed, x, prec="fp32")
    tau = 0.5 * float(np.min(np.abs(vals)))
    np.testing.assert_array_equal(gi[np.abs(gv) >= tau], oi[np.abs(ov) >= tau])
    common, ia, ib = np.intersect1d(gi, oi, return_indices=True)
    assert common.size >= np.sum(np.abs(ov) >= tau)
    l1 = np.abs(gv[ia].real - ov[ib].real) + np.abs(gv[ia].imag - ov[ib].imag)
    assert float(np.max(l1)) <= FP32_L1, float(np.max(l1))
    if v == 2:
        np.testing.assert_array_equal(gi, oi)   # v2 writes every comb candidate


def test_dense_exec_matches_oracle(S, oracle_lib):
    from sfft_gb300 import signals
    n, k, seed = 1 << 16, 50, 0
    x, _, _ = signals.make_signal(n, k, seed)
    op = oracle_lib.OraclePlan(n, k, 0)
    oi, ov = op.exec(x, seed=seed)
    ref = np.zeros(n, dtype=np.complex128)
    ref[oi] = ov
    p = S.sfft(n, k, 1)
    oracle_lib.seed_libc(seed)
    out = p.execute(x)
    np.testing.assert_array_equal(out, ref)


def test_exec_many_matches_sequential_oracle(S, oracle_lib):
    from sfft_gb300 import signals
    n, k = 1 << 16, 50
    xs = [signals.make_signal(n, k, s)[0] for s in range(5)]
    op = oracle_lib.OraclePlan(n, k, 1)
    oracle_lib.seed_libc(77)
    refs = []
    for x in xs:
        oi, ov = op.exec(x)
        r = np.zeros(n, dtype=np.complex128)
        r[oi] = ov
        refs.append(r)
    p = S.sfft(n, k, 2, max_batch=4)       # two launches: 4 + 1 signals
    oracle_lib.seed_libc(77)
    outs = p.execute_many(xs)
    for o, r in zip(outs, refs):
        np.testing.assert_array_equal(o, r)


def test_device_batch_api(S, oracle_lib):
    import ctypes
    import torch
    from sfft_gb300 import _lib, signals
    n, k, v = 1 << 16, 50, 2
    xs = [signals.make_signal(n, k, 30 + s)[0] for s in range(3)]
    op = oracle_lib.OraclePlan(n, k, v - 1)
    oracle_lib.seed_libc(5)
    refs = [op.exec(x) for x in xs]
    p = S.sfft(n, k, v)
    dev = [torch.from_numpy(x).cuda() for x in xs]
    cap = p.capacity
    oidx = torch.empty((3, cap), dtype=torch.int32, device="cuda")
    oval = torch.empty((3, cap), dtype=torch.complex128, device="cuda")
    ocnt = torch.empty(3, dtype=torch.int32, device="cuda")
    ptrs = (ctypes.c_void_p * 3)(*[t.data_ptr() for t in dev])
    oracle_lib.seed_libc(5)
    L = _lib.load()
    rc = L.sfft_exec_batch(p.sfft_plan, 3, ptrs, _lib.SFFT_IN_C128, oidx.data_ptr(), oval.data_ptr(),
                           ocnt.data_ptr(), cap, None)
    assert rc == 0, _lib.last_error()
    assert L.sfft_sync(p.sfft_plan) == 0, _lib.last_error()
    for s in range(3):
        c = int(ocnt[s])
        gi, gv = _sorted(oidx[s, :c].cpu().numpy(), oval[s, :c].cpu().numpy())
        np.testing.assert_array_equal(gi, refs[s][0])
        np.testing.assert_array_equal(gv, refs[s][1])


def test_binding_mirrors_reference_modtest(S):
    """python/test/modtest.py of the reference, in Python 3: real unit
    coefficients, every large frequency recovered within 0.1."""
    n, k = 16384, 50
    rng = np.random.default_rng(1)
    freq = rng.integers(0, n, k)
    a = np.zeros(n, dtype=complex)
    a[freq] = 1.0
    b = np.fft.ifft(a) * n
    result = S.sfft(n, k, 1).execute(b)
    for f in np.nonzero(np.abs(a) > 0.1)[0]:
        assert np.abs(result[f]) != 0.0
        assert np.abs(result[f] - a[f]) <= 0.1
