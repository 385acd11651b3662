"""The continuous-batching server (sfft_server_*): results of requests that
run in a mixed stream are identical to the same requests run alone; FP64
v1/v2 results equal the oracle's under the same seed; a small device-memory
budget still completes every request (by evicting idle plans and deferring
batches); (n, k) outside the reference's domain run with tuned constants."""
import ctypes
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env(oracle_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sfft_gb300 import _lib, build
    build.build()
    return torch, _lib, _lib.load(), oracle_lib


def _server(L, _lib, **kw):
    o = _lib.ServerOptions(-1, kw.get("max_batch", 8), kw.get("budget", 0), kw.get("k_round", 0),
                           kw.get("tune_invalid", 0))
    s = L.sfft_server_create(ctypes.byref(o))
    assert s, _lib.last_error()
    return s


def _wait(L, _lib, s, rid, cap):
    idx = np.empty(cap, dtype=np.int32)
    val = np.empty(cap, dtype=np.complex128)
    lat = ctypes.c_double()
    c = L.sfft_server_wait(s, rid, idx.ctypes.data, val.ctypes.data, cap, ctypes.byref(lat))
    assert c >= 0, _lib.last_error()
    o = np.argsort(idx[:c], kind="stable")
    return idx[:c][o], val[:c][o], lat.value


REQS = [  # (n, k, version, precision, seed)
    (1 << 16, 50, 1, 0, 1), (1 << 16, 50, 2, 0, 2), (1 << 16, 50, 2, 1, 3), (1 << 16, 50, 3, 0, 4),
    (1 << 18, 100, 2, 0, 5), (1 << 18, 100, 3, 0, 6), (1 << 16, 50, 1, 1, 7), (1 << 17, 64, 2, 1, 8),
]


def test_same_alone_and_in_the_mix(env):
    torch, _lib, L, O = env
    from sfft_gb300 import signals
    xs = {r: torch.from_numpy(signals.make_signal(r[0], r[1], r[4])[0]).cuda() for r in REQS}
    cap = 1 << 20
    # alone: one server per request
    alone = {}
    for r in REQS:
        s = _server(L, _lib)
        rid = L.sfft_server_submit(s, r[0], r[1], r[2] - 1, r[3], ctypes.c_void_p(xs[r].data_ptr()), 0, r[4])
        alone[r] = _wait(L, _lib, s, rid, cap)
        L.sfft_server_destroy(s)
    # mixed: every request three times, interleaved, waited from another thread
    s = _server(L, _lib, max_batch=4)
    ids = []
    for rep in range(3):
        for r in REQS:
            ids.append((r, L.sfft_server_submit(s, r[0], r[1], r[2] - 1, r[3], ctypes.c_void_p(xs[r].data_ptr()),
                                                0, r[4])))
    results = []
    t = threading.Thread(target=lambda: results.extend((r, _wait(L, _lib, s, i, cap)) for r, i in ids))
    t.start()
    t.join()
    stats = (ctypes.c_long * 8)()
    L.sfft_server_stats(s, stats, 8)
    L.sfft_server_destroy(s)
    assert len(results) == 3 * len(REQS)
    for r, (gi, gv, lat) in results:
        np.testing.assert_array_equal(gi, alone[r][0])
        if r[2] < 3:
            np.testing.assert_array_equal(gv, alone[r][1])     # v1/v2: identical
        else:   # v3 peels with FP64 atomics: the order of subtractions varies
            assert np.max(np.abs(gv - alone[r][1])) <= 1e-10 * max(1.0, np.max(np.abs(gv)))
        assert lat > 0
    assert stats[0] >= len(set((r[0], r[1], r[2], r[3]) for r in REQS))   # batches
    # FP64 v1/v2 requests equal the oracle seeded the same way
    for r in REQS:
        if r[2] < 3 and r[3] == 0:
            x = xs[r].cpu().numpy()
            oi, ov = O.OraclePlan(r[0], r[1], r[2] - 1).exec(x, seed=r[4])
            np.testing.assert_array_equal(alone[r][0], oi)
            np.testing.assert_array_equal(alone[r][1], ov)


def test_small_budget_evicts_and_defers(env):
    torch, _lib, L, O = env
    from sfft_gb300 import signals
    shapes = [(1 << 16, 50, 2), (1 << 17, 50, 2), (1 << 18, 50, 1)]
    xs = [torch.from_numpy(signals.make_signal(n, k, 9)[0]).cuda() for n, k, _ in shapes]
    need = max(L.sfft_server_plan_bytes(n, k, v - 1, 0, 2) for n, k, v in shapes)
    # just above the largest admission estimate: a cached plan (charged its
    # actual footprint) plus the next plan's estimate never fit together
    s = _server(L, _lib, max_batch=2, budget=int(1.05 * need))
    ids = [L.sfft_server_submit(s, n, k, v - 1, 0, ctypes.c_void_p(x.data_ptr()), 0, 3)
           for rep in range(2) for (n, k, v), x in zip(shapes, xs)]
    counts = [_wait(L, _lib, s, i, 1 << 20)[0].size for i in ids]
    stats = (ctypes.c_long * 8)()
    L.sfft_server_stats(s, stats, 8)
    L.sfft_server_destroy(s)
    assert all(c > 0 for c in counts)
    assert stats[2] > 0            # plans evicted to stay inside the budget
    assert stats[5] <= stats[6]    # bytes held <= budget


def test_tuned_constants_outside_reference_domain(env):
    torch, _lib, L, O = env
    from sfft_gb300 import signals
    from sfft_gb300.sfft import describe_plan
    n, k = 1 << 16, 200                      # the reference's v2 plan has < 2k+1 buckets
    with pytest.raises(ValueError):
        describe_plan(n, k, 2)
    x, pos, vals = signals.make_signal(n, k, 17)
    s = _server(L, _lib, tune_invalid=1)
    rid = L.sfft_server_submit(s, n, k, 1, 0, ctypes.c_void_p(torch.from_numpy(x).cuda().data_ptr()), 0, 17)
    gi, gv, _ = _wait(L, _lib, s, rid, 1 << 20)
    L.sfft_server_destroy(s)
    est = np.zeros(n, dtype=complex)
    est[gi] = np.conj(gv)
    assert np.max(np.abs(est[pos] - vals)) < 0.05   # every tone recovered (the autotuner's bar)


def test_batch_never_evicts_its_own_plan(env):
    """Two cached plans and a budget with room for both but not for a batch
    as well: a batch for the least recently used plan must evict the other
    plan, never its own (which it is about to run on)."""
    torch, _lib, L, O = env
    from sfft_gb300 import signals
    shapes = [(1 << 16, 50, 2), (1 << 17, 50, 2)]
    xs = [torch.from_numpy(signals.make_signal(n, k, 21)[0]).cuda() for n, k, _ in shapes]
    need = [L.sfft_server_plan_bytes(n, k, v - 1, 0, 2) for n, k, v in shapes]
    alone = []
    for (n, k, v), x in zip(shapes, xs):
        s = _server(L, _lib, max_batch=2)
        alone.append(_wait(L, _lib, s, L.sfft_server_submit(s, n, k, v - 1, 0, ctypes.c_void_p(x.data_ptr()), 0, 5),
                           1 << 20))
        L.sfft_server_destroy(s)
    s = _server(L, _lib, max_batch=2, budget=int(1.05 * (need[0] + need[1])))
    got = []
    for rep in range(3):
        for j, ((n, k, v), x) in enumerate(zip(shapes, xs)):
            rid = L.sfft_server_submit(s, n, k, v - 1, 0, ctypes.c_void_p(x.data_ptr()), 0, 5)
            got.append((j, _wait(L, _lib, s, rid, 1 << 20)))
    stats = (ctypes.c_long * 8)()
    L.sfft_server_stats(s, stats, 8)
    L.sfft_server_destroy(s)
    for j, (gi, gv, _) in got:
        np.testing.assert_array_equal(gi, alone[j][0])
        np.testing.assert_array_equal(gv, alone[j][1])
    assert stats[5] <= stats[6]


def test_in_order_waits_complete_when_results_fill_the_budget(env):
    """Many requests submitted at once under a budget that holds the plans
    but not all the batches' results, then waited for in submission order:
    finished, uncollected results move to host memory so that earlier
    requests are still admitted, and every result equals the request run
    alone."""
    torch, _lib, L, O = env
    from sfft_gb300 import signals
    shapes = [(1 << 16, 50, 2), (1 << 17, 50, 2)]
    xs = [torch.from_numpy(signals.make_signal(n, k, 31)[0]).cuda() for n, k, _ in shapes]
    need = [L.sfft_server_plan_bytes(n, k, v - 1, 0, 2) for n, k, v in shapes]
    alone = []
    for (n, k, v), x in zip(shapes, xs):
        s = _server(L, _lib, max_batch=2)
        alone.append(_wait(L, _lib, s, L.sfft_server_submit(s, n, k, v - 1, 0, ctypes.c_void_p(x.data_ptr()), 0, 9),
                           1 << 20))
        L.sfft_server_destroy(s)
    s = _server(L, _lib, max_batch=2, budget=int(1.3 * (need[0] + need[1])))
    order = [j for _ in range(12) for j in (0, 1)]
    ids = [L.sfft_server_submit(s, shapes[j][0], shapes[j][1], shapes[j][2] - 1, 0,
                                ctypes.c_void_p(xs[j].data_ptr()), 0, 9) for j in order]
    got = [_wait(L, _lib, s, i, 1 << 20) for i in ids]
    stats = (ctypes.c_long * 9)()
    L.sfft_server_stats(s, stats, 9)
    L.sfft_server_destroy(s)
    for j, (gi, gv, _) in zip(order, got):
        np.testing.assert_array_equal(gi, alone[j][0])
        np.testing.assert_array_equal(gv, alone[j][1])
    assert stats[5] <= stats[6]
