"""Loading of the golden records made by tests/golden/make_golden.py."""
import glob
import json
import os

import numpy as np

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NPML_REF = {"2o": 50, "iso": 20, "vti": 20, "tti": 40}


def golden_files():
    return sorted(glob.glob(os.path.join(GOLDEN_DIR, "*.npz")))


def load(path):
    z = np.load(path)
    case = json.loads(str(z["case"]))
    models = {k: z[k] for k in ("vel", "rho", "eps", "del", "theta", "phi") if k in z.files}
    out = {"rec": z["rec"]}
    if "rec_mute" in z.files:
        out["rec_mute"] = z["rec_mute"]
    return case, models, out


def mute_consistent(g_rec, g_mute, o_mute, o_rec):
    """The reference zeroed exactly the samples the candidate zeroed."""
    must_zero = (g_mute == 0) & (g_rec != 0)
    kept = g_mute != 0
    return bool(np.all(o_mute[must_zero] == 0) and np.all(o_mute[kept] == o_rec[kept]))
