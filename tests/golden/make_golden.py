"""Generate the golden fixtures from the unmodified sFFT 0.1 reference.

Runs here only (it needs the reference sources, compiled by
`make -C oracle ref` into oracle/_ref/ against this project's FFT shim):

    python tests/golden/make_golden.py            # all cases
    python tests/golden/make_golden.py c1 v3_small

For each case it stores, in tests/golden/<case>.npz: the workload (n, k,
version, seeds, magnitude law, SNR), the drawn spectrum (so the input can
be rebuilt), the plan parameters the reference computed, samples and
checksums of its filters, its output (support and values, or checksums of
them for large outputs) and, for v1/v2, its vote counts.  The reference is
executed with glibc random()/drand48() seeded by srandom(s); srand48(s).
A second, FMA-contracting build with the reference's own flags
(-O3 -ffast-math -march=native) is run on the same input and its
agreement with the portable build is recorded as `fast_*` fields.
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O            # noqa: E402
from sfft_gb300 import signals as S       # noqa: E402

# name: (version 0/1/2, n, k, signal seed, magnitudes, snr_db, exec seed, full output?)
CASES = {
    "v1_n8192_k50": (0, 8192, 50, 3, None, None, 3, True),
    "c1_v1_n65536_k50": (0, 65536, 50, 0, None, None, 0, True),
    "v1_n65536_k50_s5": (0, 65536, 50, 5, None, None, 5, True),
    "v1_n4194304_k100": (0, 1 << 22, 100, 11, None, None, 11, True),
    "v2_n65536_k50": (1, 65536, 50, 0, None, None, 0, True),
    "v2_n65536_k50_snr40": (1, 65536, 50, 2, None, 40.0, 2, True),
    "v2_n1048576_k50": (1, 1 << 20, 50, 4, None, None, 4, True),
    "c4_v2_n4194304_k100": (1, 1 << 22, 100, 7, (0.1, 10.0), 20.0, 7, False),
    "v3_n65536_k50": (2, 65536, 50, 1, None, None, 1, True),
    "v3_n262144_k100": (2, 1 << 18, 100, 1, None, None, 1, True),
    "v3_n16384_k8_early": (2, 1 << 14, 8, 21, None, None, 21, True),
    "c2_v3_n16777216_k1000": (2, 1 << 24, 1000, 1, None, None, 1, True),
}


def checksums(idx, val):
    return dict(count=int(idx.size), idx_sum=int(np.sum(idx.astype(np.int64))),
                idx_sq=float(np.sum(idx.astype(np.float64) ** 2)),
                re_sum=float(np.sum(val.real)), im_sum=float(np.sum(val.imag)),
                abs_sum=float(np.sum(np.abs(val))))


def run_case(name, spec, ref, ref_fast):
    version, n, k, sseed, mag, snr, xseed, full = spec
    x, pos, vals = S.make_signal(n, k, sseed, mag=mag, snr_db=snr)
    t0 = time.time()
    plan = ref.plan(n, k, version)
    params = ref.params(plan)
    filt = ref.filters(plan, n)
    out = ref.exec(plan, x, seed=xseed)
    t1 = time.time()
    idx = np.nonzero(out)[0].astype(np.int32)
    val = out[idx]
    rec = dict(meta=json.dumps(dict(name=name, version=version, n=n, k=k, signal_seed=sseed,
                                    mag=mag, snr_db=snr, exec_seed=xseed, full=full)),
               params=json.dumps({kk: int(v) for kk, v in params.items()}),
               spectrum_pos=pos, spectrum_val=vals,
               signal_sum=np.array([np.sum(x)]))
    for w, (t, fr) in enumerate(filt):
        rec[f"filter{w}_time_head"] = t[:16]
        rec[f"filter{w}_time_mid"] = t[t.size // 2 - 8:t.size // 2 + 8]
        rec[f"filter{w}_time_sum"] = np.array([np.sum(t), np.sum(np.abs(t))])
        rec[f"filter{w}_freq_head"] = fr[:16]
        rec[f"filter{w}_freq_sum"] = np.array([np.sum(fr), np.sum(np.abs(fr))])
    rec["checksums"] = json.dumps(checksums(idx, val))
    if full:
        rec["out_idx"] = idx
        rec["out_val"] = val
    else:
        # a deterministic sample of the support: every 97th entry
        rec["out_idx_sample"] = idx[::97]
        rec["out_val_sample"] = val[::97]
    if version < 2:
        sc = ref.score(plan, n)
        nz = np.nonzero(sc)[0].astype(np.int32)
        if full and n <= (1 << 20):
            rec["score_idx"] = nz
            rec["score_val"] = sc[nz].astype(np.int16)
        rec["score_hist"] = np.bincount(sc, minlength=16)[:16].astype(np.int64)
        rec["score_weighted"] = np.array([int(np.sum(nz.astype(np.int64) * sc[nz]))])
    ref.free(plan)
    # agreement of the reference's own fast-math build on the same input
    fplan = ref_fast.plan(n, k, version)
    fout = ref_fast.exec(fplan, x, seed=xseed)
    ref_fast.free(fplan)
    fidx = np.nonzero(fout)[0]
    same = np.array_equal(fidx, idx)
    scale = max(1.0, float(np.max(np.abs(val)))) if val.size else 1.0
    rec["fast_support_equal"] = np.array([same])
    rec["fast_max_abs_diff"] = np.array([float(np.max(np.abs(fout[idx] - val)) / scale)
                                         if same and val.size else -1.0])
    rec["fast_support_symdiff"] = np.array([len(set(fidx.tolist()) ^ set(idx.tolist()))])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **rec)
    print(f"{name}: nnz={idx.size} ref {t1 - t0:.2f}s fast_support_equal={same} "
          f"fast_maxdiff={rec['fast_max_abs_diff'][0]:.3g}", flush=True)


def main(argv):
    names = argv or list(CASES)
    O.build_ref()
    ref = O.RefLib("libsfft_ref.so")
    ref_fast = O.RefLib("libsfft_ref_fast.so")
    for name in names:
        run_case(name, CASES[name], ref, ref_fast)


if __name__ == "__main__":
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    main(sys.argv[1:])
