"""Signals of different (n, k, version, precision) in one batch
(sfft_mixed_*): the first call runs directly and captures a CUDA graph,
later calls replay it.  Every signal's result equals the same signal run
alone through its own plan with the same seed (bit-identical for v1/v2;
v3 peels with FP64 atomics, so values agree to 1e-10), replays with the
same seeds repeat the first call, and shapes outside the reference's
domain run with tuned constants."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

V1, V2, V3 = 0, 1, 2          # enum sfft_version
FP64, FP32 = 0, 1

SIGS = [  # (n, k, version, precision)
    (1 << 16, 50, V1, FP64), (1 << 16, 50, V1, FP64), (1 << 16, 50, V2, FP32),
    (1 << 17, 64, V2, FP64), (1 << 16, 50, V3, FP64), (1 << 18, 100, V2, FP32),
    (1 << 16, 50, V2, FP64), (1 << 17, 64, V2, FP64), (1 << 16, 50, V3, FP64),
    (1 << 16, 200, V2, FP64),   # fewer than 2k+1 buckets in the reference's table
]
TUNED = {9}


@pytest.fixture(scope="module")
def env(oracle_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sfft_gb300 import _lib, build
    build.build()
    return torch, _lib, _lib.load(), oracle_lib


class _Dev:
    """A device buffer owned by the library, seen by torch."""

    def __init__(self, ptr, count, typestr):
        self.__cuda_array_interface__ = {"shape": (count,), "typestr": typestr, "data": (ptr, False),
                                         "version": 3}


def _fetch(torch, ptr, count, typestr):
    if count == 0:
        return np.empty(0, dtype=np.dtype(typestr))
    return torch.as_tensor(_Dev(ptr, count, typestr), device="cuda").cpu().numpy()


def _result(torch, _lib, L, m, s):
    idx, val = ctypes.c_void_p(), ctypes.c_void_p()
    vb, cap = ctypes.c_int(), ctypes.c_long()
    c = L.sfft_mixed_result(m, s, ctypes.byref(idx), ctypes.byref(val), ctypes.byref(vb), ctypes.byref(cap))
    assert c >= 0, _lib.last_error()
    assert c <= cap.value
    i = _fetch(torch, idx.value, c, "<i4")
    f = _fetch(torch, val.value, 2 * c, "<f8" if vb.value == 16 else "<f4").astype(np.float64)
    v = f[0::2] + 1j * f[1::2]
    o = np.argsort(i, kind="stable")
    return i[o], v[o]


def _alone(torch, _lib, L, sig, x, seed):
    n, k, ver, prec = sig
    o = _lib.Options(prec, -1, 1)
    p = L.sfft_make_plan_ex(n, k, ver, 0, ctypes.byref(o))
    assert p, _lib.last_error()
    cap = L.sfft_output_capacity(p)
    d_idx = torch.empty(cap, dtype=torch.int32, device="cuda")
    d_val = torch.empty(cap, dtype=torch.complex64 if (prec == FP32 and ver != V3) else torch.complex128,
                        device="cuda")
    d_cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    ins = (ctypes.c_void_p * 1)(x.data_ptr())
    seeds = (ctypes.c_uint * 1)(seed)
    torch.cuda.synchronize()
    assert L.sfft_exec_batch_ex(p, 1, ins, 0, seeds, ctypes.c_void_p(d_idx.data_ptr()),
                                ctypes.c_void_p(d_val.data_ptr()), ctypes.c_void_p(d_cnt.data_ptr()), cap,
                                None) == 0, _lib.last_error()
    assert L.sfft_sync(p) == 0, _lib.last_error()
    c = int(d_cnt.item())
    i = d_idx[:c].cpu().numpy()
    v = d_val[:c].cpu().numpy().astype(np.complex128)
    L.sfft_free_plan(p)
    o = np.argsort(i, kind="stable")
    return i[o], v[o]


def _create(L, _lib, sigs):
    num = len(sigs)
    arr = lambda j: (ctypes.c_int * num)(*[s[j] for s in sigs])
    m = L.sfft_mixed_create(num, arr(0), arr(1), arr(2), arr(3), 0, 1, -1)
    assert m, _lib.last_error()
    return m


def _run(L, _lib, m, xs, seeds):
    num = len(xs)
    ins = (ctypes.c_void_p * num)(*[x.data_ptr() for x in xs])
    sd = (ctypes.c_uint * num)(*seeds)
    assert L.sfft_mixed_exec(m, ins, sd) == 0, _lib.last_error()
    assert L.sfft_mixed_sync(m) == 0, _lib.last_error()


def test_mixed_graph_equals_alone(env):
    torch, _lib, L, O = env
    from sfft_gb300 import signals
    sigs = [signals.make_signal(n, k, 100 + i) for i, (n, k, _, _) in enumerate(SIGS)]
    xs = [torch.from_numpy(x).cuda() for x, _, _ in sigs]
    seeds_a = [11 + i for i in range(len(SIGS))]
    seeds_b = [501 + 7 * i for i in range(len(SIGS))]
    m = _create(L, _lib, SIGS)
    assert L.sfft_mixed_groups(m) == len(set(SIGS))
    first, second, third = [], [], []
    for seeds, store in ((seeds_a, first), (seeds_b, second), (seeds_a, third)):
        _run(L, _lib, m, xs, seeds)
        store.extend(_result(torch, _lib, L, m, s) for s in range(len(SIGS)))
    L.sfft_mixed_destroy(m)
    for s, sig in enumerate(SIGS):
        exact = sig[2] != V3
        # a graph replay with the first call's seeds repeats the first call
        np.testing.assert_array_equal(third[s][0], first[s][0])
        if exact:
            np.testing.assert_array_equal(third[s][1], first[s][1])
        else:
            assert np.max(np.abs(third[s][1] - first[s][1]), initial=0) <= 1e-10 * max(
                1.0, np.max(np.abs(first[s][1]), initial=0))
        if s in TUNED:      # tuned constants: every tone recovered (the autotuner's bar)
            _, pos, vals = sigs[s]
            for gi, gv in (first[s], second[s]):
                est = np.zeros(sig[0], dtype=complex)
                est[gi] = np.conj(gv)
                assert np.max(np.abs(est[pos] - vals)) < 0.05
            continue
        # both the directly run call and the replayed call equal the signal alone
        for got, seeds in ((first[s], seeds_a), (second[s], seeds_b)):
            ai, av = _alone(torch, _lib, L, sig, xs[s], seeds[s])
            np.testing.assert_array_equal(got[0], ai)
            if exact:
                np.testing.assert_array_equal(got[1], av)
            else:
                assert np.max(np.abs(got[1] - av), initial=0) <= 1e-10 * max(1.0, np.max(np.abs(av), initial=0))
    # FP64 v1/v2 in the replayed call equal the oracle seeded the same way
    for s, sig in enumerate(SIGS):
        if s not in TUNED and sig[2] != V3 and sig[3] == FP64:
            oi, ov = O.OraclePlan(sig[0], sig[1], sig[2]).exec(sigs[s][0], seed=seeds_b[s])
            np.testing.assert_array_equal(second[s][0], oi)
            np.testing.assert_array_equal(second[s][1], ov)


def test_mixed_rejects_bad_shapes(env):
    torch, _lib, L, O = env
    bad = [(1 << 16, 50, V2, FP64), (3000, 50, V2, FP64)]      # n not a power of two
    num = len(bad)
    arr = lambda j: (ctypes.c_int * num)(*[s[j] for s in bad])
    assert not L.sfft_mixed_create(num, arr(0), arr(1), arr(2), arr(3), 0, 1, -1)
    assert _lib.last_error()


def _uneven_shapes(count, seed0=0):
    """(n, k) of an uneven v2 batch: n log-uniform over 2^16..2^22, k uniform
    in [10, 500] (the bench's uneven workload, fewer signals)."""
    out = []
    for s in range(seed0, seed0 + count):
        r = np.random.default_rng(s)
        out.append((1 << int(r.integers(16, 23)), int(r.integers(10, 501))))
    return out


def _create_tuned(L, _lib, sigs, persistent, in_type=0):
    num = len(sigs)
    arr = lambda j: (ctypes.c_int * num)(*[s[j] for s in sigs])
    m = L.sfft_mixed_create(num, arr(0), arr(1), arr(2), arr(3), in_type, 2, -1)
    assert m, _lib.last_error()
    if persistent:
        assert L.sfft_mixed_set_persistent(m, 1) == 0, _lib.last_error()
    return m


def test_persistent_executor_equals_graph(env):
    """The persistent executor (one kernel over a device work queue) must
    give every FP32 v2 signal exactly the result of the per-plan graph
    branches -- the same arithmetic per candidate -- on the direct first call
    and on graph replays, and the groups it does not take (v1, v3, FP64)
    still run as branches of the same graph."""
    torch, _lib, L, O = env
    from sfft_gb300 import signals
    shapes = _uneven_shapes(24, seed0=40)
    sigs = [(n, k, V2, FP32) for n, k in shapes]
    sigs += [(1 << 16, 50, V1, FP64), (1 << 16, 50, V3, FP64), (1 << 17, 64, V2, FP64),
             (1 << 22, 500, V2, FP32), (1 << 16, 500, V2, FP32)]   # comb of 16384; 16 candidates per residue
    data = [signals.make_signal_torch(n, k, 900 + i, snr_db=40.0) for i, (n, k, _, _) in enumerate(sigs)]
    xs = [x for x, _, _ in data]
    torch.cuda.synchronize()
    mg = _create_tuned(L, _lib, sigs, False)
    mp = _create_tuned(L, _lib, sigs, True)
    for call, seeds in enumerate(([3 + i for i in range(len(sigs))], [77 + 5 * i for i in range(len(sigs))])):
        before = L.sfft_kernel_launches()
        _run(L, _lib, mp, xs, seeds)
        launches_p = L.sfft_kernel_launches() - before
        before = L.sfft_kernel_launches()
        _run(L, _lib, mg, xs, seeds)
        launches_g = L.sfft_kernel_launches() - before
        if call == 0:
            # the direct first call: the executor plus the branches of the three
            # groups it does not take, against a branch per group
            assert launches_p < launches_g / 3, (launches_p, launches_g)
        for s, sig in enumerate(sigs):
            gi, gv = _result(torch, _lib, L, mg, s)
            pi, pv = _result(torch, _lib, L, mp, s)
            np.testing.assert_array_equal(pi, gi, err_msg=f"call {call}, signal {s} {sig}")
            if sig[2] == V3:
                assert np.max(np.abs(pv - gv), initial=0) <= 1e-10 * max(1.0, np.max(np.abs(gv), initial=0))
            else:
                np.testing.assert_array_equal(pv, gv, err_msg=f"call {call}, signal {s} {sig}")
    L.sfft_mixed_destroy(mg)
    L.sfft_mixed_destroy(mp)


def test_persistent_executor_alone_is_one_launch(env):
    """An all-FP32 v2 batch runs as exactly one kernel launch per call."""
    torch, _lib, L, O = env
    from sfft_gb300 import signals
    sigs = [(n, k, V2, FP32) for n, k in _uneven_shapes(12, seed0=7)]
    xs = [signals.make_signal_torch(n, k, 300 + i, snr_db=40.0)[0] for i, (n, k, _, _) in enumerate(sigs)]
    torch.cuda.synchronize()
    m = _create_tuned(L, _lib, sigs, True)
    before = L.sfft_kernel_launches()
    _run(L, _lib, m, xs, list(range(len(sigs))))
    assert L.sfft_kernel_launches() - before == 1
    _run(L, _lib, m, xs, list(range(len(sigs))))     # a graph replay
    for s, (n, k, _, _) in enumerate(sigs):
        gi, gv = _result(torch, _lib, L, m, s)
        assert gi.size > 0
    L.sfft_mixed_destroy(m)


def test_persistent_executor_complex64_inputs(env):
    """complex64 inputs (the executor's other instantiation) give the same
    results through the executor as through the graph branches."""
    torch, _lib, L, O = env
    from sfft_gb300 import signals
    sigs = [(n, k, V2, FP32) for n, k in _uneven_shapes(10, seed0=70)]
    xs = [signals.make_signal_torch(n, k, 500 + i, snr_db=40.0)[0].to(torch.complex64)
          for i, (n, k, _, _) in enumerate(sigs)]
    torch.cuda.synchronize()
    mg = _create_tuned(L, _lib, sigs, False, in_type=1)
    mp = _create_tuned(L, _lib, sigs, True, in_type=1)
    seeds = [9 + i for i in range(len(sigs))]
    _run(L, _lib, mg, xs, seeds)
    _run(L, _lib, mp, xs, seeds)
    for s in range(len(sigs)):
        gi, gv = _result(torch, _lib, L, mg, s)
        pi, pv = _result(torch, _lib, L, mp, s)
        np.testing.assert_array_equal(pi, gi)
        np.testing.assert_array_equal(pv, gv)
    L.sfft_mixed_destroy(mg)
    L.sfft_mixed_destroy(mp)
