"""The FP64 estimation's division (host reciprocal, one correction, exact
remainder certificate, IEEE fallback) returns exactly the IEEE quotient:
checked against the device's IEEE division on pseudo-random operands with
exponents near 1 and across most of the double range."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def L():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sfft_gb300 import _lib, build
    build.build()
    return _lib.load()


@pytest.mark.parametrize("span,count", [(4, 1 << 26), (60, 1 << 26), (500, 1 << 25)])
def test_certified_division_equals_ieee(L, span, count):
    cert = ctypes.c_long()
    bad = L.sfft_selftest_division(12345 + span, count, span, ctypes.byref(cert))
    assert bad == 0
    if span <= 60:
        assert cert.value > 0.9 * count      # the fast path carries almost every division
