"""Synthetic k-sparse test signals (the role of src/simulation.cc:95-112).

The reference draws k frequencies with replacement, magnitude 1, phase 0,
and builds x with an unnormalised backward FFT (src/simulation.cc:103-111).
The workloads here draw k distinct frequencies uniformly, magnitudes 1.0 or
log-uniform, phases uniform in [0, 2 pi), optionally add complex white
Gaussian noise at a given SNR, and also use the unnormalised backward
transform x[t] = sum_f X[f] exp(+2 pi i f t / n), so that sFFT returns X.

numpy (host) and torch (device) variants draw the same spectrum for the same
seed; the time signal is computed by numpy's or torch's FFT respectively.
"""
import numpy as np


def sparse_spectrum(n, k, seed, mag=None):
    """k distinct frequencies of [0, n) with values.

    mag: None for |X| = 1, or (lo, hi) for log-uniform magnitudes.
    Returns (positions int64 sorted by draw order, values complex128).
    """
    rng = np.random.default_rng(seed)
    pos = []
    seen = set()
    while len(pos) < k:
        for f in rng.integers(0, n, size=2 * (k - len(pos)) + 8):
            f = int(f)
            if f not in seen:
                seen.add(f)
                pos.append(f)
                if len(pos) == k:
                    break
    phase = rng.random(k) * (2.0 * np.pi)
    if mag is None:
        m = np.ones(k)
    else:
        lo, hi = mag
        m = np.exp(rng.uniform(np.log(lo), np.log(hi), size=k))
    return np.asarray(pos, dtype=np.int64), m * np.exp(1j * phase)


def noise_sigma(x_power, snr_db):
    """Per-component std of complex AWGN for mean signal power x_power."""
    p_noise = x_power / (10.0 ** (snr_db / 10.0))
    return np.sqrt(p_noise / 2.0)


def time_signal(n, pos, vals, snr_db=None, noise_seed=0):
    """x = n * ifft(X) (+ complex AWGN at snr_db), complex128."""
    X = np.zeros(n, dtype=np.complex128)
    X[pos] = vals
    x = np.fft.ifft(X) * n
    if snr_db is not None:
        rng = np.random.default_rng(noise_seed + 0x9E3779B9)
        sig = noise_sigma(np.mean(np.abs(x) ** 2), snr_db)
        x = x + sig * (rng.standard_normal(n) + 1j * rng.standard_normal(n))
    return np.ascontiguousarray(x)


def make_signal(n, k, seed, mag=None, snr_db=None):
    """Convenience: (x, positions, values) for one seeded workload."""
    pos, vals = sparse_spectrum(n, k, seed, mag)
    return time_signal(n, pos, vals, snr_db, noise_seed=seed), pos, vals


def make_signal_torch(n, k, seed, mag=None, snr_db=None, device="cuda", dtype=None):
    """Device-side variant for large batches (torch FFT on the GPU)."""
    import torch
    pos, vals = sparse_spectrum(n, k, seed, mag)
    X = torch.zeros(n, dtype=torch.complex128, device=device)
    X[torch.as_tensor(pos, device=device)] = torch.as_tensor(vals, device=device)
    x = torch.fft.ifft(X) * n
    if snr_db is not None:
        g = torch.Generator(device=device)
        g.manual_seed(int(seed) + 0x9E3779B9)
        p = float(torch.mean(torch.abs(x) ** 2))
        sig = float(noise_sigma(p, snr_db))
        nr = torch.randn(n, generator=g, device=device, dtype=torch.float64)
        ni = torch.randn(n, generator=g, device=device, dtype=torch.float64)
        x = x + sig * torch.complex(nr, ni)
    if dtype is not None:
        x = x.to(dtype)
    return x.contiguous(), pos, vals
