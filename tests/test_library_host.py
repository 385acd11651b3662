"""Host-side checks of the C-ABI library that need no GPU: it builds, loads,
exports every function include/sfft.h declares, fails loudly without a
device, and computes plans identical to the reference's (via the oracle)."""
import ctypes

import numpy as np
import pytest

from sfft_gb300 import _lib, build


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def test_exports_every_declared_symbol(lib):
    names = _lib.header_functions()
    for required in ("sfft_malloc", "sfft_free", "sfft_make_plan", "sfft_free_plan", "sfft_exec",
                     "sfft_exec_many"):
        assert required in names
    for name in names:
        assert hasattr(lib, name), name


def test_plan_struct_layout_matches_reference():
    # src/sfft.h:44-50: {sfft_version version; unsigned n, k; void *data;}
    assert ctypes.sizeof(_lib.Plan) == 24
    assert _lib.Plan.data.offset == 16


def test_malloc_is_aligned_and_freeable(lib):
    p = lib.sfft_malloc(1 << 20)
    assert p and p % 16 == 0
    lib.sfft_free(p)
    lib.sfft_free(None)


def test_no_device_means_no_plan(lib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    plan = lib.sfft_make_plan(1 << 16, 50, 0, _lib.FFTW_ESTIMATE)
    assert not plan
    assert "CUDA" in _lib.last_error()


def test_invalid_arguments_rejected(lib):
    assert not lib.sfft_make_plan(1000, 50, 0, _lib.FFTW_ESTIMATE)        # not a power of two
    assert _lib.last_error()
    assert not lib.sfft_make_plan(1 << 16, 50, 7, _lib.FFTW_ESTIMATE)     # no such version
    f = (ctypes.c_long * 11)()
    assert lib.sfft_describe_plan(1 << 14, 4, 2, f, 11) == -1              # v3 needs k >= 8
    assert lib.sfft_describe_plan(8192, 1000, 0, f, 11) == -1              # B < 2k+1


PLAN_CASES = [(8192, 50, 1), (1 << 16, 50, 1), (1 << 16, 50, 2), (1 << 18, 100, 2), (1 << 20, 50, 2),
              (1 << 16, 50, 3), (1 << 18, 100, 3), (1 << 14, 8, 3), (4000, 100, 1)]


@pytest.mark.parametrize("n,k,v", [c for c in PLAN_CASES if c[0] & (c[0] - 1) == 0])
def test_plans_identical_to_oracle(lib, oracle_lib, n, k, v):
    from sfft_gb300 import sfft as S
    op = oracle_lib.OraclePlan(n, k, v - 1)
    mine = S.describe_plan(n, k, v)
    for key, val in mine.items():
        assert op.params[key] == val, key
    for which in (0, 1):
        t, f = S.describe_filter(n, k, v, which)
        np.testing.assert_array_equal(t, op.filter_time(which))
        np.testing.assert_array_equal(f, op.filter_freq(which))


def test_tuned_constants_lookup(lib):
    """k buckets, and table-or-rule constants that always leave at least
    2k+1 buckets (the algorithm's domain) for v1/v2 shapes."""
    from sfft_gb300 import _lib
    assert [lib.sfft_tuned_k(k) for k in (1, 16, 17, 100, 500, 512, 513)] == [16, 16, 32, 128, 512, 512, 1024]
    import ctypes
    import math
    for n in (1 << 16, 1 << 19, 1 << 22):
        for k in (10, 100, 500):
            for v in (0, 1):
                p = _lib.Params()
                src = lib.sfft_tuned_params(n, k, v, ctypes.byref(p))
                assert src in (0, 1)
                s = math.sqrt(n * k / math.log2(n))
                B = 1 << int(math.floor(math.log2(p.Bcst_loc * s)))
                assert B >= 2 * k + 1
                assert 1 <= p.threshold_loops <= p.loc_loops and p.est_loops >= 1
    assert lib.sfft_tuned_params(1 << 16, 10, 2, ctypes.byref(_lib.Params())) == -1   # v3: none


def _median_network(lib, n):
    buf = np.zeros(3 * 512, dtype=np.int32)
    c = lib.sfft_debug_median_network(n, buf.ctypes.data, buf.size)
    assert c > 0
    return buf[:3 * c].reshape(c, 3)


@pytest.mark.parametrize("n", list(range(8, 25)))
def test_median_networks_exhaustive(lib, n):
    """Every compiled lower-median selection network, on all 2^n inputs of
    0s and 1s: a network of min/max operations selects the m-th smallest
    of any n values iff it does so for every 0-1 input (min and max commute
    with monotone maps).  Element (n-1)/2 of the output must be 1 exactly
    when at least n - (n-1)/2 inputs are 1."""
    net = _median_network(lib, n)
    m = (n - 1) // 2
    chunk = 1 << min(n, 20)
    for base in range(0, 1 << n, chunk):
        x = np.arange(base, base + chunk, dtype=np.uint32)
        v = [((x >> np.uint32(w)) & np.uint32(1)).astype(bool) for w in range(n)]
        ones = np.zeros(chunk, dtype=np.int32)
        for w in range(n):
            ones += v[w]
        for i, j, kind in net:
            if kind == 1:
                v[i], v[j] = v[i] & v[j], v[i] | v[j]
            elif kind == 2:
                v[i] = v[i] & v[j]
            else:
                assert kind == 3
                v[j] = v[i] | v[j]
        np.testing.assert_array_equal(v[m], ones >= n - m)


def test_median_network_sizes(lib):
    """The pruned pairwise networks: fewer min/max operations than the
    pruned merge-exchange networks they replaced (143 for n = 20)."""
    ops = {n: int(sum(2 if k == 1 else 1 for _, _, k in _median_network(lib, n))) for n in (8, 12, 16, 20, 24)}
    assert ops[20] == 125, ops
    assert ops == {8: 27, 12: 53, 16: 87, 20: 125, 24: 169}, ops
    assert lib.sfft_debug_median_network(7, None, 0) == -1
