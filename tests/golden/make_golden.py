"""Generate the golden records that pin the CPU oracle to the reference.

Run on a machine with a GPU, from the repository root, after the reference's
kernels were built into oracle/_ref/ by oracle/build_ref.sh (on a machine that
has the reference sources):

    make -C oracle harness
    python tests/golden/make_golden.py --out /tmp/golden

Each case seeds a small smooth model (numpy default_rng + Gaussian smoothing),
writes it in the reference's raw float32 format, runs the reference's own CUDA
kernels through oracle/_build/refharness, and stores the models, the case
parameters and the reference's full record rec[iy, ix, it] in <name>.npz (before the
direct-wave mute; cases with mute=1 also store the muted record as rec_mute).  The
models are stored, so the tests never depend on the random generator's stream.

Case constraints that follow from the reference code:
  * 2nd order: the padded size nn = n + 108 satisfies nn % 16 in {0, 12..15}, so
    the sponge kernel's unguarded tail threads (Toa_3dfd_cuda.cu:123-154) only
    touch the never-updated outer 4-cell margin.
  * VTI/TTI: ny <= nx, because the reference sizes its y PML arrays by nnx
    (..vti..:503-510, ..tti..:516-523).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

CASES = [
    dict(name="2o_a", engine="2o", nx=20, ny=20, nz=20, sx=10, sy=9, sz=5, nt=200, dt=1e-3,
         fm=25.0, mute=1, seed=11),
    dict(name="iso_a", engine="iso", nx=20, ny=18, nz=16, sx=9, sy=8, sz=4, nt=250, dt=1e-3,
         fm=25.0, wtype=1, mute=1, seed=12),
    dict(name="iso_w2", engine="iso", nx=12, ny=12, nz=12, sx=5, sy=6, sz=3, nt=150, dt=1e-3,
         fm=30.0, wtype=2, seed=21),
    dict(name="iso_w3", engine="iso", nx=12, ny=12, nz=12, sx=5, sy=6, sz=3, nt=150, dt=1e-3,
         fm=30.0, wtype=3, seed=22),
    dict(name="iso_w4", engine="iso", nx=12, ny=12, nz=12, sx=5, sy=6, sz=3, nt=150, dt=1e-3,
         fm=30.0, wtype=4, seed=23),
    dict(name="iso_w5", engine="iso", nx=12, ny=12, nz=12, sx=5, sy=6, sz=3, nt=150, dt=1e-3,
         fm=30.0, wtype=5, seed=24),
    dict(name="iso_w6", engine="iso", nx=12, ny=12, nz=12, sx=5, sy=6, sz=3, nt=150, dt=1e-3,
         fm=30.0, wtype=6, seed=25),
    dict(name="vti_a", engine="vti", nx=20, ny=18, nz=16, sx=9, sy=8, sz=4, nt=250, dt=1e-3,
         fm=25.0, mute=1, seed=13),
    dict(name="tti_a", engine="tti", nx=20, ny=18, nz=16, sx=9, sy=8, sz=4, nt=250, dt=1e-3,
         fm=25.0, mute=1, seed=14),
]

MODELS = {"2o": ("vel",), "iso": ("vel", "rho"), "vti": ("vel", "rho", "eps", "del"),
          "tti": ("vel", "eps", "del", "theta", "phi")}


def smooth_field(rng, shape, lo, hi, sigma=2.0):
    """Seeded smooth field in [lo, hi]; shape is (ny, nx, nz) (z fastest on disk)."""
    from scipy.ndimage import gaussian_filter
    a = gaussian_filter(rng.standard_normal(shape), sigma=sigma, mode="reflect")
    a = (a - a.min()) / max(a.max() - a.min(), 1e-12)
    return (lo + (hi - lo) * a).astype(np.float32)


def make_models(case):
    rng = np.random.default_rng(case["seed"])
    shape = (case["ny"], case["nx"], case["nz"])
    vel = smooth_field(rng, shape, 1800.0, 3000.0)
    m = {"vel": vel, "rho": (310.0 * vel.astype(np.float64) ** 0.25).astype(np.float32)}
    eps = smooth_field(rng, shape, 0.05, 0.25)
    m["eps"] = eps
    m["del"] = np.minimum(smooth_field(rng, shape, 0.0, 0.12), eps).astype(np.float32)
    # gently varying angles: the reference's TTI update grows without bound where
    # the azimuth varies quickly (its rotated derivatives are not energy-conserving)
    m["theta"] = smooth_field(rng, shape, 0.0, 0.4, sigma=4.0)
    m["phi"] = smooth_field(rng, shape, 0.2, 0.8, sigma=4.0)
    return {k: m[k] for k in MODELS[case["engine"]]}


def write_case(case, models, d):
    with open(os.path.join(d, "case.txt"), "w") as f:
        for k in ("engine", "nx", "ny", "nz", "sx", "sy", "sz", "nt", "dt", "fm"):
            f.write(f"{k} {case[k]}\n")
        f.write("dx 10\ndy 10\ndz 10\n")
        f.write(f"wtype {case.get('wtype', 1)}\nmute {case.get('mute', 0)}\n")
    for k, a in models.items():
        a.tofile(os.path.join(d, f"{k}.bin"))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--harness", default="oracle/_build/refharness")
    ap.add_argument("--cubins", default="oracle/_ref")
    args = ap.parse_args()
    os.makedirs(args.out, exist_ok=True)
    for case in CASES:
        models = make_models(case)
        with tempfile.TemporaryDirectory() as d:
            write_case(case, models, d)
            r = subprocess.run([args.harness, args.cubins, d], capture_output=True, text=True)
            sys.stdout.write(r.stdout)
            sys.stderr.write(r.stderr)
            if r.returncode != 0:
                raise SystemExit(f"harness failed on {case['name']}")
            shape = (case["ny"], case["nx"], case["nt"])
            out = {"rec": np.fromfile(os.path.join(d, "rec_ref.bin"), np.float32).reshape(shape)}
            if case.get("mute", 0):
                out["rec_mute"] = np.fromfile(os.path.join(d, "rec_mute.bin"),
                                              np.float32).reshape(shape)
        rec = out["rec"]
        np.savez_compressed(os.path.join(args.out, case["name"] + ".npz"),
                            case=json.dumps(dict(case, dx=10.0, dy=10.0, dz=10.0)), **out, **models)
        print(case["name"], "max|rec| =", float(np.abs(rec).max()))


if __name__ == "__main__":
    main()
