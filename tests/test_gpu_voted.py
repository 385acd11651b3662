"""The opt-in v2 voted mode (sfft_plan_v2_voted): only candidates that reach
the vote threshold are estimated.  Each of them gets exactly the value the
full (reference) mode gives it under the same draws, every tone of a
noiseless signal is among them, and the list is far shorter."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sfft_gb300 import _lib, build
    build.build()
    return torch, _lib, _lib.load()


def _exec(torch, _lib, L, p, xs, seeds, prec):
    cap = L.sfft_output_capacity(p)
    num = len(xs)
    idx = torch.empty((num, cap), dtype=torch.int32, device="cuda")
    val = torch.empty((num, cap), dtype=torch.complex128 if prec == 0 else torch.complex64, device="cuda")
    cnt = torch.zeros(num, dtype=torch.int32, device="cuda")
    ins = (ctypes.c_void_p * num)(*[x.data_ptr() for x in xs])
    sd = (ctypes.c_uint * num)(*seeds)
    torch.cuda.synchronize()
    assert L.sfft_exec_batch_ex(p, num, ins, 0, sd, ctypes.c_void_p(idx.data_ptr()), ctypes.c_void_p(val.data_ptr()),
                                ctypes.c_void_p(cnt.data_ptr()), cap, None) == 0, _lib.last_error()
    assert L.sfft_sync(p) == 0, _lib.last_error()
    out = []
    for s in range(num):
        c = int(cnt[s])
        i = idx[s, :c].cpu().numpy()
        v = val[s, :c].cpu().numpy()
        o = np.argsort(i, kind="stable")
        out.append((i[o], v[o]))
    return out


@pytest.mark.parametrize("n,k,prec", [(1 << 18, 100, 0), (1 << 22, 100, 0), (1 << 22, 100, 1)])
def test_voted_values_equal_full_mode(env, n, k, prec):
    torch, _lib, L = env
    from sfft_gb300 import signals
    sig = [signals.make_signal_torch(n, k, 40 + s) for s in range(3)]
    xs = [x for x, _, _ in sig]
    seeds = [5, 6, 7]
    o = _lib.Options(prec, -1, 3)
    p = L.sfft_make_plan_ex(n, k, 1, 0, ctypes.byref(o))
    assert p, _lib.last_error()
    full = _exec(torch, _lib, L, p, xs, seeds, prec)
    assert L.sfft_plan_v2_voted(p, 1) == 0, _lib.last_error()
    voted = _exec(torch, _lib, L, p, xs, seeds, prec)
    assert L.sfft_plan_v2_voted(p, 0) == 0, _lib.last_error()
    again = _exec(torch, _lib, L, p, xs, seeds, prec)
    L.sfft_free_plan(p)
    for s in range(3):
        fi, fv = full[s]
        vi, vv = voted[s]
        assert 0 < vi.size < fi.size // 10
        pos = np.searchsorted(fi, vi)
        assert np.all(fi[pos] == vi)                        # a subset of the full list
        np.testing.assert_array_equal(vv, fv[pos])          # with the same values
        _, tones, vals = sig[s]
        est = np.zeros(n, dtype=complex)
        est[vi] = np.conj(vv.astype(np.complex128))
        assert np.max(np.abs(est[tones] - vals)) < (1e-6 if prec == 0 else 1e-3)   # every tone
        np.testing.assert_array_equal(again[s][0], fi)      # back to the reference's list
        np.testing.assert_array_equal(again[s][1], fv)


def test_voted_mode_only_for_v2(env):
    torch, _lib, L = env
    o = _lib.Options(0, -1, 1)
    p = L.sfft_make_plan_ex(1 << 16, 50, 0, 0, ctypes.byref(o))
    assert p, _lib.last_error()
    assert L.sfft_plan_v2_voted(p, 1) == -1
    L.sfft_free_plan(p)
