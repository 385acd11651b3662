"""Loading of the golden fixtures in tests/golden (made by make_golden.py)."""
import glob
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)
    d = {k: z[k] for k in z.files}
    d["meta"] = json.loads(str(d["meta"]))
    d["params"] = json.loads(str(d["params"]))
    d["checksums"] = json.loads(str(d["checksums"]))
    return d


def signal(g):
    """Rebuild the fixture's input from its stored spectrum (and noise seed)."""
    from sfft_gb300 import signals as S
    m = g["meta"]
    return S.time_signal(m["n"], g["spectrum_pos"], g["spectrum_val"], m["snr_db"],
                         noise_seed=m["signal_seed"])
