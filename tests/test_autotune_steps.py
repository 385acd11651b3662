"""The autotuner's search steps (host-only): a step of the location bucket
count keeps the comb width W = Comb_cst n / B_loc (a narrower comb let tone
pairs cancel in a shared class), only the comb knob moves W, loop counts
stay at the rule's, and the Python rule equals the library's."""
import ctypes

import pytest

from sfft_gb300 import _lib
from sfft_gb300.autotune import KNOBS, rule_params, step


def _plan(L, n, k, d):
    f = (ctypes.c_long * 11)()
    p = _lib.Params(**d)
    m = L.sfft_describe_plan_params(n, k, 1, ctypes.byref(p), f, 11)
    return None if m < 0 else {"B_loc": f[0], "B_est": f[2], "W": f[3], "L_loc": f[5], "L_est": f[7]}


@pytest.mark.parametrize("n,k", [(1 << 18, 512), (1 << 21, 512), (1 << 22, 100), (1 << 16, 32)])
def test_bucket_steps_keep_the_comb_width(n, k):
    L = _lib.load()
    d = rule_params(n, k)
    base = _plan(L, n, k, d)
    assert base is not None
    for up in (True, False):
        e = step(d, "B_loc", up, 1)
        p = _plan(L, n, k, e)
        if p is None:      # outside the domain (fewer than 2k+1 buckets)
            continue
        assert p["B_loc"] == base["B_loc"] * (2 if up else 1) // (1 if up else 2)
        assert p["W"] == base["W"]
    e = step(d, "comb", True, 1)
    assert _plan(L, n, k, e)["W"] == 2 * base["W"]


def test_loop_counts_are_not_searched():
    assert set(KNOBS) == {"B_loc", "B_est", "comb"}


@pytest.mark.parametrize("n,k", [(1 << 16, 16), (1 << 20, 128), (1 << 22, 512), (1 << 23, 100)])
def test_python_rule_equals_the_library_rule(n, k):
    L = _lib.load()
    p = _lib.Params()
    src = L.sfft_tuned_params(n, k, 1, ctypes.byref(p))
    if src == 1:
        pytest.skip("a table row exists for this shape")
    r = rule_params(n, k)
    for f, _ in p._fields_:
        assert getattr(p, f) == r[f], f
