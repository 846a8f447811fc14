"""Generate the full-size golden records: the reference's own CUDA kernels on the
benchmark workloads at their full sizes.

Run on a machine with a GPU, from the repository root, after the reference's
kernels were built into oracle/_ref/ (oracle/build_ref.sh, on a machine that has
the reference sources) and the harness was built (make -C oracle harness):

    python tests/golden/make_golden_full.py --out tests/golden/full

Workloads (bench.workload, seeded synthetic models; the reference's compiled
absorber widths):
  2o128   2nd order, 128^3 three-layer model, nt 1000, 50-cell sponge, record at z 1
  iso256  1st-order isotropic, 256^3 smooth model, Gardner density, nt 2000, PML 20
  vti384  VTI, 384 x 384 x 256 smooth fields, nt 2500, PML 20
  tti256  TTI, 256^3 smooth fields (tilt 0-45 deg, azimuth 0-360 deg), nt 3000, PML 40

A full record is 0.07-1.5 GB, so each <name>.npz keeps:
  rec        the unmuted record at every J-th receiver line in x and y, starting
             at the shot's own line (J = 16 for 128 cells, 32 otherwise), all samples
  zeroed, kept  packed bit masks over those traces: samples the reference's mute
             zeroed (muted 0, unmuted not 0), and samples it left alone (muted not 0)
  trace_norm the L2 norm of every trace of the full unmuted record, [ny][nx]
  model_sha256  of the model arrays the workload generator produced (the tests
             regenerate the models and check this first)
  ref_loop_ms   the harness's CUDA-event time of the reference's time loop
  ref_vs_fp64   (with --fp64) relative L2 of the reference's full unmuted record
             against the same shot run by this build's FP64 engine: how far the
             reference's own FP32 arithmetic lies from the FP64 solution
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

WORKLOADS = ("2o128", "iso256", "vti384", "tti256")


def model_sha256(models):
    h = hashlib.sha256()
    for k in sorted(models):
        h.update(k.encode())
        h.update(np.ascontiguousarray(models[k], np.float32).tobytes())
    return h.hexdigest()


def trace_lines(n, s, step):
    """Receiver lines s mod step, s mod step + step, ... below n."""
    return np.arange(s % step, n, step)


def step_for(n):
    return 16 if n <= 128 else 32


def write_case(d, cfgd, models, shot, mute, sync=1):
    with open(os.path.join(d, "case.txt"), "w") as f:
        f.write(f"engine {cfgd['physics']}\nnx {cfgd['nx']}\nny {cfgd['ny']}\nnz {cfgd['nz']}\n")
        f.write(f"dx {cfgd['dx']}\ndy {cfgd['dy']}\ndz {cfgd['dz']}\n")
        f.write(f"sx {shot[0]}\nsy {shot[1]}\nsz {shot[2]}\nnt {cfgd['nt']}\n")
        f.write(f"dt {cfgd['dt']!r}\nfm {cfgd['fm']}\nwtype 1\nmute {int(mute)}\nsync {int(sync)}\n")
    for k, a in models.items():
        np.ascontiguousarray(a, np.float32).tofile(os.path.join(d, f"{k}.bin"))


def run_harness(cfgd, models, shot, harness, cubins, mute=True, sync=1):
    """(unmuted record [ny][nx][nt], muted record or None, loop ms)"""
    with tempfile.TemporaryDirectory() as d:
        write_case(d, cfgd, models, shot, mute, sync)
        r = subprocess.run([harness, cubins, d], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"refharness failed ({r.returncode}): {r.stderr.strip()}")
        ms = float(r.stdout.split("ms=")[1].split()[0])
        shape = (cfgd["ny"], cfgd["nx"], cfgd["nt"])
        rec = np.fromfile(os.path.join(d, "rec_ref.bin"), np.float32).reshape(shape)
        recm = np.fromfile(os.path.join(d, "rec_mute.bin"), np.float32).reshape(shape) if mute else None
    return rec, recm, ms


def summarise(rec, recm, shot, nx, ny):
    iy = trace_lines(ny, shot[1], step_for(ny))
    ix = trace_lines(nx, shot[0], step_for(nx))
    sel = np.ix_(iy, ix)
    r, m = rec[sel], recm[sel]
    return dict(iy=iy.astype(np.int32), ix=ix.astype(np.int32), rec=np.ascontiguousarray(r),
                zeroed=np.packbits((m == 0) & (r != 0)), kept=np.packbits(m != 0),
                trace_norm=trace_norms(rec))


def trace_norms(rec):
    """L2 norm of every trace [ny][nx] (float64 sums, one receiver line at a time)."""
    return np.stack([np.linalg.norm(rec[i].astype(np.float64), axis=1) for i in range(rec.shape[0])]).astype(
        np.float32)


def fp64_distance(cfgd, models, shot, rec):
    """relative L2 of rec against the same shot run by the FP64 engine"""
    sys.path.insert(0, os.path.join(ROOT, "acoustic3d-fd_gb300"))
    import a3d
    cfg = a3d.make_config(cfgd["physics"], cfgd["nx"], cfgd["ny"], cfgd["nz"], dx=cfgd["dx"], dy=cfgd["dy"],
                          dz=cfgd["dz"], nt=cfgd["nt"], dt=cfgd["dt"], fm=cfgd["fm"], npml=cfgd["npml"],
                          rec_z=cfgd.get("rec_z", -1), storage=a3d.FP64)
    e = a3d.Engine(cfg, models)
    try:
        r64 = e.run(*shot)
    finally:
        e.close()
    num = sum(float(np.sum((rec[i].astype(np.float64) - r64[i]) ** 2)) for i in range(rec.shape[0]))
    den = sum(float(np.sum(r64[i].astype(np.float64) ** 2)) for i in range(rec.shape[0]))
    return (num / den) ** 0.5


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "full"))
    ap.add_argument("--harness", default=os.path.join(ROOT, "oracle", "_build", "refharness"))
    ap.add_argument("--cubins", default=os.path.join(ROOT, "oracle", "_ref"))
    ap.add_argument("--only", nargs="*", default=list(WORKLOADS))
    ap.add_argument("--fp64", action="store_true", help="also store the reference's distance from an FP64 run")
    args = ap.parse_args()
    import bench
    os.makedirs(args.out, exist_ok=True)
    for name in args.only:
        t0 = time.time()
        cfgd, models, shot, meta = bench.workload(name)
        rec, recm, ms = run_harness(cfgd, models, shot, args.harness, args.cubins)
        s = summarise(rec, recm, shot, cfgd["nx"], cfgd["ny"])
        del recm
        case = dict(workload=name, **cfgd, shot=list(shot), meta=meta, ref_loop_ms=ms)
        if args.fp64:
            s["ref_vs_fp64"] = np.float64(fp64_distance(cfgd, models, shot, rec))
        np.savez_compressed(os.path.join(args.out, name + ".npz"), case=json.dumps(case),
                            model_sha256=model_sha256(models), **s)
        print(f"{name}: reference loop {ms:.1f} ms, max|rec| {float(np.abs(rec).max()):.4g}, "
              f"{time.time() - t0:.1f} s", flush=True)


if __name__ == "__main__":
    main()
