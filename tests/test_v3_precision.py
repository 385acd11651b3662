"""Why v3 has no FP32 form, measured: at the C2 shape (n = 2^24, k = 1000)
an FP32 Gaussian filter (fold and bucket FFT in single precision, decoded in
FP64) mislocates a large share of the tones the FP64 filter locates, while
an FP32 Mansour comb decodes exactly the same frequencies.

The Gaussian decode of estimate_freq_gauss_loops2
(computefourier-3.0.cc:484-640) takes the full frequency from the phase
difference of the two time shifts, freq = round(n / 2 pi * (d1 - d0)), which
needs phase errors well below pi / n = 1.9e-7 rad; FP32 bucket values carry
relative errors of about 1e-7.  The Mansour decode
(estimate_freq_mansour_loops2, :642-776) keeps only the high bits
(freq & ~(W - 1)) of the same expression, so it needs pi W / n.

The buckets of the first Gaussian filter and of the Mansour comb are formed
here in numpy from the oracle's plan (filter taps, random offsets of one
exec), once in FP64 and once with FP32 inputs, taps, products, sums and FFT,
and decoded with the reference's tests in FP64.  A third test bounds the
difference between the permuted filter's phase factors as the reference
forms them (a running product) and as the GPU does (power tables)."""
import numpy as np
import pytest

N, K, SEED = 1 << 24, 1000, 11


@pytest.fixture(scope="module")
def setup(oracle_lib):
    sfft = pytest.importorskip("scipy.fft")
    from sfft_gb300 import signals
    x, pos, _ = signals.make_signal(N, K, SEED)
    op = oracle_lib.OraclePlan(N, K, 2)
    oracle_lib.seed_libc(SEED)
    op.exec(x)
    return sfft, x, pos, op, op.params, op.v3_debug()


def _gauss_buckets(sfft, x, taps, B, w, g, dt):
    chunks = w // B
    T = chunks * B
    xx, tt = x.astype(dt), taps[:T].astype(dt)
    out = []
    for l in (0, 1):
        prod = (xx[(g + l + np.arange(T)) % N] * tt).reshape(chunks, B)
        s = np.zeros(B, dtype=dt)
        for c in range(chunks):  # the reference's order: chunk by chunk
            s = s + prod[c]
        out.append(sfft.fft(s).astype(np.complex128))
    return out


def _gauss_decode(u, B):
    a0, b0, a1, b1 = u[0].real, u[0].imag, u[1].real, u[1].imag
    c0, c1 = a0 * a0 + b0 * b0, a1 * a1 + b1 * b1
    err = (c1 / np.where(c0 > 0, c0, 1) - 1) ** 2 / N
    freq = (np.rint(N / (2 * np.pi) * (np.arctan2(b1, a1) - np.arctan2(b0, a0))).astype(np.int64) + N) & (N - 1)
    hashed = np.rint(freq * B / N).astype(np.int64) & (B - 1)
    ok = (c0 + c1 > 1e-8) & (err < 1e-12) & (c0 > 0.01) & (hashed == np.arange(B))
    return ok, freq


def _mansour(sfft, x, W, io, dt):
    sigma = N // W
    return [sfft.fft(x[(io + l + np.arange(W) * sigma) % N].astype(dt)).astype(np.complex128) for l in (0, 1)]


def _mansour_decode(u, W, io):
    norm = 1.0 / W
    a0, b0, a1, b1 = u[0].real, u[0].imag, u[1].real, u[1].imag
    c0, c1 = (a0 * a0 + b0 * b0) * norm * norm, (a1 * a1 + b1 * b1) * norm * norm
    d0, d1 = np.arctan2(b0 * norm, a0 * norm), np.arctan2(b1 * norm, a1 * norm)
    e = (c1 / np.where(c0 > 0, c0, 1) - 1) ** 2
    ok = (c0 + c1 > 1e-8) & (e < N * 1e-10) & (c0 > 0.01)
    f1 = np.rint((d1 - d0) * N / (2 * np.pi)).astype(np.int64)
    f3 = (f1 & ((N - 1) & ~(W - 1))) | np.arange(W)
    val = np.sqrt(c0) * np.exp(1j * (d0 - 2 * np.pi / N * ((f3 * io) % N)))
    return ok, f3, val


def test_fp32_gaussian_filter_mislocates_tones(setup):
    sfft, x, pos, op, p, dbg = setup
    B, w, g = p["B_g1"], p["w_g1"], dbg["init_G_offset"]
    taps = op.filter_time(0)
    ok64, f64 = _gauss_decode(_gauss_buckets(sfft, x, taps, B, w, g, np.complex128), B)
    ok32, f32 = _gauss_decode(_gauss_buckets(sfft, x, taps, B, w, g, np.complex64), B)
    right64 = ok64 & np.isin(f64, pos)
    right32 = ok32 & np.isin(f32, pos)
    lost = int(np.sum(right64 & ~right32))
    moved = int(np.sum(ok64 & ok32 & (f64 != f32)))
    print(f"Gaussian filter, C2: FP64 locates {int(right64.sum())} tones in {int(ok64.sum())} decoded buckets; "
          f"FP32 loses {lost} of them, {moved} decoded frequencies differ")
    assert right64.sum() >= 40                 # the FP64 decode finds tones (55 at this seed)
    assert lost >= 0.2 * right64.sum()         # FP32 loses a large share of them (22 of 55)
    assert moved >= 0.1 * ok64.sum()           # and moves many decoded frequencies (85 of 296)


def test_fp32_mansour_comb_decodes_the_same(setup):
    sfft, x, pos, op, p, dbg = setup
    W, io = p["W_Man"], dbg["init_offset"]
    ok64, f64, v64 = _mansour_decode(_mansour(sfft, x, W, io, np.complex128), W, io)
    ok32, f32, v32 = _mansour_decode(_mansour(sfft, x, W, io, np.complex64), W, io)
    both = ok64 & ok32
    assert np.array_equal(ok64, ok32)
    assert np.array_equal(f64[both], f32[both])
    assert int(np.sum(both & np.isin(f64, pos))) >= 800   # the comb locates most tones (881 of 1000)
    rel = np.abs(v64[both] - v32[both]) / np.abs(v64[both])
    assert float(np.max(rel)) < 1e-6


def test_phase_power_tables_match_the_running_product(setup):
    """The permuted Gaussian's phase factors: the reference forms shift_i by
    the running product shift_{i+1} = shift_i * step (computefourier-3.0.cc:
    66-87); the GPU forms (shift_0 step^(LO hi)) step^lo from two tables
    built by binary powering (FP64, separately rounded complex products).
    At the C2 shape both stay within 1e-12 of each other (the chain's own
    rounding drift), far inside the 1e-10 value tolerance."""
    _, _, _, op, p, dbg = setup
    ig, ai, b = dbg["init_G_offset"], dbg["ai"], dbg["b"]
    count = (p["w_g2"] // p["B_g2"]) * p["B_g2"] + 1
    a0, a1 = 2 * np.pi * ig * b / N, 2 * np.pi * ai * b / N   # the reference's angles
    sh0, st = complex(np.cos(a0), np.sin(a0)), complex(np.cos(a1), np.sin(a1))
    chain = np.empty(count, dtype=np.complex128)
    sh = sh0
    for i in range(count):
        chain[i] = sh
        sh = sh * st

    def cpow(a, e):
        r = 1 + 0j
        while e:
            if e & 1:
                r = r * a
            e >>= 1
            if e:
                a = a * a
        return r

    lo = 1
    while lo * lo < count:
        lo *= 2
    hi = (count + lo - 1) // lo
    t_lo = [cpow(st, e) for e in range(lo)]
    s_lo = cpow(st, lo)
    t_hi = [sh0 * cpow(s_lo, h) for h in range(hi)]
    tab = np.array([t_hi[i // lo] * t_lo[i % lo] for i in range(count)])
    assert float(np.max(np.abs(tab - chain))) < 1e-12
