"""Pin the CPU oracle to the unmodified reference: every golden fixture in
tests/golden was produced by the reference (built against the FFT shim) and
the oracle must reproduce its plan, filters, vote counts and output."""
import numpy as np
import pytest

import golden_cases as G

CASES = G.names()


def _check_outputs(g, idx, val):
    m = g["meta"]
    keep = val != 0
    idx, val = idx[keep], val[keep]
    cs = g["checksums"]
    assert idx.size == cs["count"]
    assert int(np.sum(idx.astype(np.int64))) == cs["idx_sum"]
    if "out_idx" in g:
        np.testing.assert_array_equal(idx, g["out_idx"])
        ref_val = g["out_val"]
    else:
        pos = np.searchsorted(idx, g["out_idx_sample"])
        np.testing.assert_array_equal(idx[pos], g["out_idx_sample"])
        val = val[pos]
        ref_val = g["out_val_sample"]
    scale = max(1.0, float(np.max(np.abs(ref_val)))) if ref_val.size else 1.0
    err = float(np.max(np.abs(val - ref_val))) / scale if ref_val.size else 0.0
    if m["version"] < 2:
        # v1/v2 perform only + - * / at exec time: bit-exact on identical inputs
        assert err <= 1e-12, err
    else:
        # v3 calls atan2/sin/cos/sqrt and iterates the result map in a
        # different order than the reference (insertion vs hash order)
        assert err <= 1e-10, err


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference(name, oracle_lib):
    g = G.load(name)
    m = g["meta"]
    if m["n"] >= (1 << 24) and not pytest.importorskip("numpy"):
        pytest.skip()
    x = G.signal(g)
    plan = oracle_lib.OraclePlan(m["n"], m["k"], m["version"])
    for key, v in g["params"].items():
        assert plan.params[key] == v, key
    for w in range(2):
        t = plan.filter_time(w)
        np.testing.assert_array_equal(t[:16], g[f"filter{w}_time_head"])
        np.testing.assert_array_equal(t[t.size // 2 - 8:t.size // 2 + 8], g[f"filter{w}_time_mid"])
        fr = plan.filter_freq(w)
        np.testing.assert_array_equal(fr[:16], g[f"filter{w}_freq_head"])
        np.testing.assert_allclose(np.sum(fr), g[f"filter{w}_freq_sum"][0], rtol=1e-12)
    idx, val = plan.exec(x, seed=m["exec_seed"])
    _check_outputs(g, idx, val)
    if m["version"] < 2:
        sc = plan.score()
        np.testing.assert_array_equal(np.bincount(sc, minlength=16)[:16], g["score_hist"])
        nz = np.nonzero(sc)[0]
        assert int(np.sum(nz.astype(np.int64) * sc[nz])) == int(g["score_weighted"][0])
        if "score_idx" in g:
            np.testing.assert_array_equal(nz, g["score_idx"])
            np.testing.assert_array_equal(sc[nz], g["score_val"])


def test_shim_fft_accuracy(oracle_lib):
    rng = np.random.default_rng(0)
    for n in [1, 2, 4, 8, 64, 1024, 4096, 8192, 3041, 11011, 22023]:
        x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        y = oracle_lib.shim_fft(x, -1)
        z = np.fft.fft(x)
        assert np.max(np.abs(y - z)) <= 2e-15 * max(1.0, np.max(np.abs(z))) * np.log2(max(n, 2))
        yb = oracle_lib.shim_fft(x, +1)
        assert np.max(np.abs(yb - np.fft.ifft(x) * n)) <= 2e-15 * max(1.0, np.max(np.abs(z))) * np.log2(max(n, 2))


def test_oracle_rejects_outside_domain(oracle_lib):
    with pytest.raises(ValueError):
        oracle_lib.OraclePlan(1000, 10, 0)        # not a power of two
    with pytest.raises(ValueError):
        oracle_lib.OraclePlan(1 << 14, 4, 2)      # v3 needs k >= 8
    with pytest.raises(ValueError):
        oracle_lib.OraclePlan(8192, 1000, 0)      # B < 2k+1
