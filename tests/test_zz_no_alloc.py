"""sfft_exec_noalloc: the transform for callers that cannot allocate GPU
memory while they run (their device memory belongs to their own pool, they
run under a fixed budget, or cudaMalloc/cudaFree would stall their stream).
Its scratch is a static array inside the library, so its result must equal
what sfft_exec_sparse (which uses the plan's allocated workspace) returns,
on consecutive calls that reuse the same array.  Kept in a file of its own
that pytest collects last."""
import ctypes

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


@pytest.mark.parametrize("version,precision", [(1, "fp64"), (2, "fp64"), (2, "fp32")])
def test_noalloc_matches_allocating_entry_point(env, version, precision):
    torch, _lib, L, O = env
    from sfft_gb300 import signals
    from sfft_gb300.sfft import sfft
    n, k = 1 << 16, 50
    plan = sfft(n, k, version, precision=precision)
    cap = plan.capacity
    vdt = torch.complex128 if precision == "fp64" else torch.complex64
    oidx = torch.empty(cap, dtype=torch.int32, device="cuda")
    oval = torch.empty(cap, dtype=vdt, device="cuda")
    status = torch.zeros(2, dtype=torch.int32, device="cuda")
    stream = torch.cuda.Stream()
    for call, seed in enumerate((11, 12)):       # two calls in a row share the scratch
        x, _, _ = signals.make_signal(n, k, seed)
        O.seed_libc(seed)
        ri, rv = plan.execute_sparse(x)          # the existing, allocating entry point
        o = np.argsort(ri)
        ri, rv = ri[o], rv[o]
        xd = torch.from_numpy(x).cuda()
        torch.cuda.synchronize()
        O.seed_libc(seed)
        rc = L.sfft_exec_noalloc(plan.sfft_plan, ctypes.c_void_p(xd.data_ptr()), _lib.SFFT_IN_C128,
                                 ctypes.c_void_p(oidx.data_ptr()), ctypes.c_void_p(oval.data_ptr()), cap,
                                 ctypes.c_void_p(status.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, _lib.last_error()
        stream.synchronize()
        cnt, err = (int(v) for v in status.cpu())
        assert err == 0, f"device error bits {err} on call {call}"
        gi = oidx[:cnt].cpu().numpy()
        gv = oval[:cnt].cpu().numpy().astype(np.complex128)
        o = np.argsort(gi)
        gi, gv = gi[o], gv[o]
        # the same tolerance as the other parity tests: both paths run the
        # same kernels on the same draws, so the results are identical
        np.testing.assert_array_equal(gi, ri)
        np.testing.assert_array_equal(gv, rv)


def _noalloc_call(env, plan, x, seed, stream):
    torch, _lib, L, O = env
    cap = plan.capacity
    vdt = torch.complex128 if plan.precision == "fp64" else torch.complex64
    oidx = torch.empty(cap, dtype=torch.int32, device="cuda")
    oval = torch.empty(cap, dtype=vdt, device="cuda")
    status = torch.zeros(2, dtype=torch.int32, device="cuda")
    xd = torch.from_numpy(x).cuda()
    torch.cuda.synchronize()
    O.seed_libc(seed)
    rc = L.sfft_exec_noalloc(plan.sfft_plan, ctypes.c_void_p(xd.data_ptr()), _lib.SFFT_IN_C128,
                             ctypes.c_void_p(oidx.data_ptr()), ctypes.c_void_p(oval.data_ptr()), cap,
                             ctypes.c_void_p(status.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    assert rc == 0, _lib.last_error()
    stream.synchronize()
    cnt, err = (int(v) for v in status.cpu())
    assert err == 0, f"device error bits {err}"
    gi = oidx[:cnt].cpu().numpy()
    gv = oval[:cnt].cpu().numpy().astype(np.complex128)
    o = np.argsort(gi)
    return gi[o], gv[o]


def test_noalloc_alternating_plans_of_different_sizes(env):
    """Plans whose scratch layouts differ, called in turn on the one shared
    array: v1 results depend on the vote counters, so a counter left by
    another plan's call that passed for one of this call's would add or
    drop a frequency.  Every call must equal the allocating entry point
    (itself bit-identical to the oracle), and the FP64 v1 calls the oracle
    directly."""
    torch, _lib, L, O = env
    from sfft_gb300 import signals
    from sfft_gb300.sfft import sfft
    shapes = [(1 << 16, 50, 1, "fp64"), (1 << 17, 64, 1, "fp32"), (1 << 18, 50, 2, "fp64"),
              (1 << 16, 50, 2, "fp32"), (1 << 18, 100, 1, "fp64"), (1 << 17, 64, 2, "fp64"),
              (1 << 17, 64, 2, "fp32")]     # FP32 v2 estimated by comb residue class
    plans = [sfft(n, k, v, precision=p) for n, k, v, p in shapes]
    stream = torch.cuda.Stream()
    order = [0, 1, 2, 0, 3, 4, 1, 6, 0, 5, 2, 4, 6, 0, 3, 1, 5, 4, 0, 2, 6, 1, 0]   # large after small and back
    for call, i in enumerate(order):
        n, k, v, p = shapes[i]
        seed = 300 + call
        x, pos, vals = signals.make_signal(n, k, seed, snr_db=30.0 if v == 2 else None)
        O.seed_libc(seed)
        ri, rv = plans[i].execute_sparse(x)
        o = np.argsort(ri)
        ri, rv = ri[o], rv[o]
        gi, gv = _noalloc_call(env, plans[i], x, seed, stream)
        np.testing.assert_array_equal(gi, ri, err_msg=f"call {call}: {shapes[i]}")
        np.testing.assert_array_equal(gv, rv, err_msg=f"call {call}: {shapes[i]}")
        if v == 1 and p == "fp64":
            oi, ov = O.OraclePlan(n, k, 0).exec(x, seed=seed)
            np.testing.assert_array_equal(gi, oi, err_msg=f"call {call}: {shapes[i]} vs the oracle")
            np.testing.assert_array_equal(gv, ov, err_msg=f"call {call}: {shapes[i]} vs the oracle")


def test_noalloc_rejects_plans_beyond_its_scratch(env):
    torch, _lib, L, O = env
    from sfft_gb300.sfft import sfft
    plan = sfft(1 << 20, 50, 1)
    buf = torch.empty(4, dtype=torch.int32, device="cuda")
    rc = L.sfft_exec_noalloc(plan.sfft_plan, ctypes.c_void_p(buf.data_ptr()), _lib.SFFT_IN_C128,
                             ctypes.c_void_p(buf.data_ptr()), ctypes.c_void_p(buf.data_ptr()), plan.capacity,
                             ctypes.c_void_p(buf.data_ptr()), None)
    assert rc == -1
    assert "static scratch" in _lib.last_error()
