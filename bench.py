#!/usr/bin/env python
"""Benchmark of the forward-modelling hot path: grid-point updates per second.

Default workload (the configuration the headline metric is quoted on): the
1st-order staggered-grid isotropic engine with density, 256^3 model, dx = 10 m,
nt = 2000, dt = 0.4*dx/vmax (CFL 0.4), velocity = Gaussian-smoothed (sigma 8
cells) N(0,1) noise from seed 2 mapped to 1500-4500 m/s, Gardner density
rho = 310 v^0.25, 20-cell PML, 20 Hz Ricker at the grid centre, depth 8,
receivers on every surface node.  FP32 wavefields.

A "step" is one shot: the full nt-step time loop over the padded grid.
  value  Gpts/s = updated cells of the padded grid x nt x shots / device time
         (CUDA events on the engine's stream around each time loop; inputs resident)
  e2e    the same metric through the host-buffer C-ABI call a3d_forward_host:
         model H2D, time loop, record D2H, every step
  roofline  the dominant kernel's algorithmic bytes per launch / its mean launch
         time (events around every launch), against the measured HBM peak
  cpu_baseline  the CPU restatement of the reference update (oracle, OpenMP, all
         host cores) on a bounded sample of the same workload
  rel_l2_vs_fp64  shot-record error of the FP32 run against the same shot run in
         FP64 (GPU FP64 path), outside the timed region

--impl reference times the reference's own implementation of the path, which is
CUDA: its four .cu files built unchanged for sm_103a into cubins (oracle/_ref, by
oracle/build_ref.sh where the reference sources are) and driven by
oracle/_build/refharness, which replays the reference's host loop with its launch
shapes and its device synchronisations; a bench step is one full shot (or, where a
shot of the reference takes longer than REF_SAMPLE_S, the first steps of it).
Where the cubins are absent it times the reference's update restated on the CPU
(the oracle's literal form, all host cores) instead, and says so.
Multi-GPU: replicas (torchrun; each rank runs its own shots, no collective in the
data path); value = all ranks' updates / max rank time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "acoustic3d-fd_gb300")
for _p in (PKG, os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

# bytes per cell of the two isotropic sweeps as built (compulsory traffic of each launch):
#   velocity sweep: read P, u, v, w, rho; write u, v, w            -> 8 words
#   stress sweep:   read u, v, w, P, rho, vp; write P              -> 7 words
# and the whole-step algorithmic figure of an unsplit formulation (u,v,w,P read and
# written once + 2 parameters): 10 words = 40 B per cell update.
#   VTI velocity: P, Q, u, v, w, 1/rho read, u, v, w written -> 9 words; stress: u, v, w,
#   P, Q, rho, vp, eps, del read, P, Q written -> 11 words
#   TTI velocity: P, Q, u, v, w + 4 trig read, u, v, w written -> 12 words; stress:
#   u, v, w, P, Q, vp, eps, del + 4 trig read, P, Q written -> 14 words
KERNEL_BYTES = {"iso": (32.0, 28.0), "2o": (16.0, None), "vti": (36.0, 44.0), "tti": (48.0, 56.0)}
STEP_BYTES = {"iso": 40.0, "2o": 16.0, "vti": 56.0, "tti": 60.0}
# 2-byte wavefield storage (isotropic and VTI engines; the model parameters stay float):
#   velocity sweep: P, u, v, w (2 B) + 1/rho (4 B) read, u, v, w written -> 18 B
#   stress sweep:   u, v, w, P (2 B) + rho, vp (4 B) read, P written     -> 18 B
#   unsplit step: (u, v, w, P) read and written at 2 B + 2 float parameters -> 24 B
#   VTI: velocity P, Q, u, v, w (2 B) + 1/rho read, u, v, w written -> 20 B; stress
#   u, v, w, P, Q (2 B) + rho, vp, eps, del read, P, Q written -> 30 B; step 36 B
KERNEL_BYTES_2B = {"iso": (18.0, 18.0), "vti": (20.0, 30.0), "tti": (32.0, 42.0)}
#   fused isotropic step (FP32): u, v, w, P, 1/rho, rho, vp read, u, v, w, P written -> 44 B
FUSED_BYTES = 44.0
#   TTI: velocity P, Q, u, v, w (2 B) + 4 trig floats read, u, v, w written -> 32 B;
#   stress u, v, w, P, Q (2 B) + vp, eps, del + 4 trig read, P, Q written -> 42 B;
#   step: (u, v, w, P, Q) read and written at 2 B + 5 float parameters -> 40 B
STEP_BYTES_2B = {"iso": 24.0, "vti": 36.0, "tti": 40.0}
# float16 u, v, w with float P, Q and split components (VTI, "fp16v"):
#   velocity: P, Q (4 B) + u, v, w (2 B) + 1/rho read, u, v, w written -> 24 B; stress:
#   u, v, w (2 B) + P, Q (4 B) + rho, vp, eps, del read, P, Q written -> 38 B; step
#   (u, v, w) read and written at 2 B, (P, Q) at 4 B, 4 float parameters -> 44 B
#   TTI: velocity P, Q (4 B) + u, v, w (2 B) + 4 trig floats read, u, v, w written
#   -> 36 B; stress u, v, w (2 B) + P, Q (4 B) + vp, eps, del + 4 trig read, P, Q
#   written -> 50 B; step (u, v, w) at 2 B, (P, Q) at 4 B, 5 float parameters -> 48 B
KERNEL_BYTES_MIXED = {"vti": (24.0, 38.0), "tti": (36.0, 50.0)}
STEP_BYTES_MIXED = {"vti": 44.0, "tti": 48.0}
STORAGE = {"fp32": 0, "bf16": 1, "fp16": 2, "fp16v": 4}


def workload(name, nt_override=None):
    if name == "iso256":
        import synthetic as S
        n, dx, vmax = 256, 10.0, 4500.0
        m = S.iso_model(n, 2, vmax)
        vel, rho = m["vel"], m["rho"]
        dt = np.float32(0.4 * dx / vmax)
        nt = nt_override or 2000
        cfg = dict(physics="iso", nx=n, ny=n, nz=n, dx=dx, dy=dx, dz=dx, nt=nt, dt=float(dt), fm=20.0,
                   npml=20)
        return cfg, {"vel": vel, "rho": rho}, (n // 2, n // 2, 8), \
            dict(workload="iso1order_256cube_nt%d" % nt, model="256x256x256", dx_m=dx, nt=nt,
                 dt_s=float(dt), npml=20, fm_hz=20.0, shot=[n // 2, n // 2, 8], storage="fp32")
    if name == "2o128":
        import synthetic as S
        n, dx = 128, 10.0
        vel = S.layered_2o(n)["vel"]
        nt = nt_override or 1000
        cfg = dict(physics="2o", nx=n, ny=n, nz=n, dx=dx, dy=dx, dz=dx, nt=nt, dt=5e-4, fm=25.0, npml=50,
                   rec_z=1)
        return cfg, {"vel": vel}, (64, 64, 5), \
            dict(workload="2order_128cube_3layer_nt%d" % nt, model="128x128x128", dx_m=dx, nt=nt, dt_s=5e-4,
                 sponge=50, fm_hz=25.0, shot=[64, 64, 5], storage="fp32")
    if name == "2o128lit":
        # the same model and shot as 2o128 in the configuration's literal form: a
        # 20-cell absorber, receivers at model depth 5, the direct-wave mute on and a
        # snapshot of the model window every 100 steps (the reference compiles in a
        # 50-cell sponge, records at depth 1, leaves its mute commented out and snaps
        # every 500 steps, so it cannot run this form)
        import synthetic as S
        n, dx = 128, 10.0
        vel = S.layered_2o(n)["vel"]
        nt = nt_override or 1000
        cfg = dict(physics="2o", nx=n, ny=n, nz=n, dx=dx, dy=dx, dz=dx, nt=nt, dt=5e-4, fm=25.0, npml=20,
                   rec_z=5, mute=True, snap_every=100)
        return cfg, {"vel": vel}, (64, 64, 5), \
            dict(workload="2order_128cube_3layer_literal_nt%d" % nt, model="128x128x128", dx_m=dx, nt=nt,
                 dt_s=5e-4, sponge=20, rec_z=5, mute=True, snap_every=100, fm_hz=25.0, shot=[64, 64, 5],
                 storage="fp32")
    if name == "vti384":
        # 384 x 384 x 256, d 12.5 m, nt 2500, 20-cell PML (the reference's compiled
        # width), smooth seeded fields: v 1500-4500 (seed 3), Gardner density,
        # epsilon 0-0.3 (seed 4), delta = min(delta', epsilon), delta' 0-0.15 (seed 5);
        # dt = 0.4 d / (vmax sqrt(1.6)), 15 Hz Ricker at (24, 24, 2)
        import synthetic as S
        nx, ny, nz, d, vmax = 384, 384, 256, 12.5, 4500.0
        m = S.vti_model(nx, ny, nz, vmax)
        vel, rho, eps, dl = m["vel"], m["rho"], m["eps"], m["del"]
        dt = np.float32(0.4 * d / (vmax * np.sqrt(1.6)))
        nt = nt_override or 2500
        cfg = dict(physics="vti", nx=nx, ny=ny, nz=nz, dx=d, dy=d, dz=d, nt=nt, dt=float(dt), fm=15.0, npml=20)
        return cfg, {"vel": vel, "rho": rho, "eps": eps, "del": dl}, (24, 24, 2), \
            dict(workload="vti1order_384x384x256_nt%d" % nt, model="384x384x256", dx_m=d, nt=nt,
                 dt_s=float(dt), npml=20, fm_hz=15.0, shot=[24, 24, 2], storage="fp32")
    if name == "tti256":
        # one 256^3 aperture of the TTI survey: d 12.5 m, nt 3000, 40-cell PML (the
        # reference's compiled width), smooth seeded fields: v 1500-5000 (seed 7),
        # epsilon 0-0.3 (seed 8), delta <= epsilon in 0-0.15 (seed 9), tilt 0-45 deg
        # (seed 10), azimuth 0-360 deg (seed 11), in radians; 15 Hz Ricker at the
        # aperture centre, z = 2
        import synthetic as S
        n, d, vmax = 256, 12.5, 5000.0
        m = S.tti_model(n, n, n, vmax)
        vel, eps, dl, th, ph = m["vel"], m["eps"], m["del"], m["theta"], m["phi"]
        dt = np.float32(0.4 * d / (vmax * np.sqrt(1.6)))
        nt = nt_override or 3000
        cfg = dict(physics="tti", nx=n, ny=n, nz=n, dx=d, dy=d, dz=d, nt=nt, dt=float(dt), fm=15.0, npml=40)
        return cfg, {"vel": vel, "eps": eps, "del": dl, "theta": th, "phi": ph}, (n // 2, n // 2, 2), \
            dict(workload="tti1order_256cube_nt%d" % nt, model="256x256x256", dx_m=d, nt=nt,
                 dt_s=float(dt), npml=40, fm_hz=15.0, shot=[n // 2, n // 2, 2], storage="fp32")
    raise SystemExit(f"unknown workload {name}")


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                rows.append((float(f[0]), float(f[1]), float(f[2]), f[3:7]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        load = [r for r in rows if r[2] > 300.0] or rows
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in load for i, v in enumerate(r[3]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in load), "sm_max_mhz": max(r[1] for r in rows),
                "samples": len(load), "reasons": reasons}


def cpu_rate(cfgd, models, shot, threads, nt_a=2, nt_b=None, target_s=10.0):
    """Oracle (the reference update on the CPU, literal arithmetic) Gpts/s from two
    runs of different length, so set-up time cancels.  nt_b defaults to the number
    of steps that takes about target_s seconds (from a calibration run)."""
    import oracle as O
    eng = cfgd["physics"]
    if nt_b is None:
        r, _ = cpu_rate(cfgd, models, shot, threads, 2, 6)
        per_step = updated_cells(cfgd) / (r * 1e9)
        nt_b = nt_a + max(4, min(2000, int(target_s / per_step)))
    times = []
    for nt in (nt_a, nt_b):
        s = O.Shot(cfgd["nx"], cfgd["ny"], cfgd["nz"], dx=cfgd["dx"], dy=cfgd["dy"], dz=cfgd["dz"],
                   sx=shot[0], sy=shot[1], sz=shot[2], nt=nt, dt=cfgd["dt"], fm=cfgd["fm"],
                   npml=cfgd["npml"], rec_z=cfgd.get("rec_z", 1), form=0, threads=threads)
        t0 = time.perf_counter()
        O.run(eng, s, models, "f32")
        times.append(time.perf_counter() - t0)
    pad = cfgd["npml"] + (4 if eng == "2o" else 0)
    cells = (cfgd["nx"] + 2 * pad - 8) * (cfgd["ny"] + 2 * pad - 8) * (cfgd["nz"] + 2 * pad - 8)
    dt = max(times[1] - times[0], 1e-9)
    return cells * (nt_b - nt_a) / dt / 1e9, dict(steps=nt_b - nt_a, seconds=dt)


def updated_cells(cfgd):
    pad = cfgd["npml"] + (4 if cfgd["physics"] == "2o" else 0)
    return (cfgd["nx"] + 2 * pad - 8) * (cfgd["ny"] + 2 * pad - 8) * (cfgd["nz"] + 2 * pad - 8)


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_per_launch(workload_name):
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    return d.get(workload_name)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def legacy_call(cfgd, paths, shotfile, shot, dev):
    """One call of the reference-facing drop-in entry point of this physics (model
    files in, decimation 1, record file out, no snapshots), as readmodel.py makes it."""
    import ctypes
    from ctypes import c_bool, c_float, c_int
    import a3d
    L = a3d.lib()
    b = lambda x: ctypes.c_char_p(x.encode())
    g = [c_int(cfgd["nx"]), c_int(cfgd["ny"]), c_int(cfgd["nz"]), c_float(cfgd["dx"]), c_float(cfgd["dy"]),
         c_float(cfgd["dz"]), c_int(shot[0]), c_int(shot[1]), c_int(shot[2]), c_int(1), c_int(1), c_int(1),
         c_float(cfgd["dx"]), c_float(cfgd["dy"]), c_float(cfgd["dt"]), c_int(cfgd["nt"])]
    tail = [c_bool(False), c_bool(False), c_int(100), c_int(dev)]
    eng, snap = cfgd["physics"], b(os.path.dirname(shotfile) + "/snap_")
    if eng == "iso":
        rc = L.cuda_3dfd_1order(b(paths["vel"]), b(paths["rho"]), snap, b(shotfile), c_int(0), c_int(1), *g,
                                c_float(cfgd["dt"]), c_int(1), c_float(cfgd["fm"]), *tail)
    elif eng == "vti":
        rc = L.cuda_3dfd_vti(b(paths["vel"]), b(paths["rho"]), b(paths["eps"]), b(paths["del"]), snap, b(shotfile),
                             c_int(0), c_int(1), *g, c_float(cfgd["dt"]), c_float(cfgd["fm"]), *tail)
    elif eng == "tti":
        rc = L.cuda_3dfd_tti(b(paths["vel"]), b(paths["vel"]), b(paths["eps"]), b(paths["del"]), b(paths["theta"]),
                             b(paths["phi"]), snap, b(shotfile), c_int(0), c_int(1), *g, c_float(cfgd["dt"]),
                             c_float(cfgd["fm"]), *tail)
    else:
        rc = L.cuda_3dfd(b(paths["vel"]), snap, b(shotfile), c_int(0), c_int(1), *g, c_int(0),
                         c_float(cfgd["dt"]), c_float(cfgd["fm"]), *tail)
    if rc != 0:
        raise RuntimeError(f"legacy entry point returned {rc}: {a3d.last_error()}")


def legacy_e2e(cfgd, models, shot, dev, reps=2):
    """Gpts/s of the drop-in entry point end to end (files in and out, in a temporary
    directory), one warm call then `reps` timed ones; None where the workload is not
    the reference's own configuration."""
    import tempfile
    if cfgd.get("snap_every") or cfgd.get("mute"):
        return None
    with tempfile.TemporaryDirectory() as d:
        paths = {}
        for k, a in models.items():
            paths[k] = os.path.join(d, k + ".bin")
            np.ascontiguousarray(a, np.float32).tofile(paths[k])
        shotfile = os.path.join(d, "shot.bin")
        legacy_call(cfgd, paths, shotfile, shot, dev)
        t0 = time.perf_counter()
        for _ in range(reps):
            legacy_call(cfgd, paths, shotfile, shot, dev)
        sec = (time.perf_counter() - t0) / reps
    return {"value": updated_cells(cfgd) * cfgd["nt"] / sec / 1e9, "unit": "Gpts/s", "seconds_per_call": sec,
            "call": {"iso": "cuda_3dfd_1order", "vti": "cuda_3dfd_vti", "tti": "cuda_3dfd_tti",
                     "2o": "cuda_3dfd"}[cfgd["physics"]] + " (model files in, record file out)"}


def bench_config(meta, cfgd, ws):
    """The line's `config`, identical in both arms: the workload description, the
    replica count and the L2 statement."""
    eng = cfgd["physics"]
    pad = cfgd["npml"] + (4 if eng == "2o" else 0)
    padded = (cfgd["nx"] + 2 * pad) * (cfgd["ny"] + 2 * pad) * ((cfgd["nz"] + 2 * pad + 7) // 8 * 8)
    nvol = {"2o": 3, "iso": 7, "vti": 11, "tti": 14}[eng]
    mb = 4 * padded * nvol // 2**20
    l2 = ("inputs larger than L2: %d MB of wavefields and model" % mb if mb > 126 else
          "working set %d MB fits the 126 MB L2 (L2-resident; a bench step is a whole shot, whose time "
          "steps reuse it, so no flush)" % mb)
    return dict(meta, parallelism=f"replicas{ws}", l2=l2)


REF_SAMPLE_S = 8.0  # longest reference time loop one bench step of the reference arm runs
REF_HARNESS = os.path.join(ROOT, "oracle", "_build", "refharness")
REF_CUBINS = os.path.join(ROOT, "oracle", "_ref")
REF_CUBIN = {"2o": "ref_2order.cubin", "iso": "ref_1order.cubin", "vti": "ref_vti.cubin", "tti": "ref_tti.cubin"}


def reference_cuda_available(eng):
    return os.path.exists(REF_HARNESS) and os.path.exists(os.path.join(REF_CUBINS, REF_CUBIN[eng]))


def run_reference_cuda(args, cfgd, models, shot, meta):
    """The reference's own CUDA kernels on this GPU: one harness run per bench step,
    loop time by CUDA events inside the harness, clocks sampled around the timed runs."""
    import tempfile
    eng = cfgd["physics"]
    cells = updated_cells(cfgd)
    nt = cfgd["nt"]
    with tempfile.TemporaryDirectory() as d:
        with open(os.path.join(d, "case.txt"), "w") as f:
            f.write(f"engine {eng}\nnx {cfgd['nx']}\nny {cfgd['ny']}\nnz {cfgd['nz']}\n")
            f.write(f"dx {cfgd['dx']}\ndy {cfgd['dy']}\ndz {cfgd['dz']}\n")
            f.write(f"sx {shot[0]}\nsy {shot[1]}\nsz {shot[2]}\nnt {nt}\n")
            f.write(f"dt {cfgd['dt']!r}\nfm {cfgd['fm']}\nwtype 1\nmute 0\nsync 1\n")
        for k, a in models.items():
            np.ascontiguousarray(a, np.float32).tofile(os.path.join(d, f"{k}.bin"))

        def once(steps):
            r = subprocess.run([REF_HARNESS, REF_CUBINS, d, str(steps)], capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"refharness failed ({r.returncode}): {r.stderr.strip()[-300:]}")
            return float(r.stdout.split("ms=")[1].split()[0])

        probe = max(1, min(nt, 50))
        per = once(probe) / probe  # ms per time step, with the reference's syncs
        steps = nt if per * nt <= REF_SAMPLE_S * 1000.0 else max(50, int(REF_SAMPLE_S * 1000.0 / per))
        for _ in range(args.warmup):
            once(steps)
        total = 0.0
        with ClockSampler(0) as clk:
            for _ in range(args.steps):
                total += once(steps)
    value = cells * steps * args.steps / (total / 1000.0) / 1e9
    return value, total, steps, clk.summary()


def run_reference(args, cfgd, models, shot, meta):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    config = bench_config(meta, cfgd, ws)
    eng = cfgd["physics"]
    if reference_cuda_available(eng):
        value, total_ms, steps, clocks = run_reference_cuda(args, cfgd, models, shot, meta)
        sample = (f"the reference's own CUDA kernels ({REF_CUBIN[eng]}: its .cu built unchanged for sm_103a) "
                  f"driven by its host loop restated in oracle/refharness.cpp, the reference's launch shapes "
                  f"and device synchronisations, {steps} of {cfgd['nt']} time steps per bench step, loop time "
                  f"by CUDA events, on this GPU")
        line = {"metric": "Gpts/s", "value": value, "unit": "Gpts/s", "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": total_ms / max(args.steps, 1),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic", "config": config, "impl": "reference",
                "reference_kind": "cuda",
                "cpu_baseline": {"value": value, "unit": "Gpts/s", "cores": 1, "kind": "reference",
                                 "sample": sample},
                "e2e": {"value": value, "unit": "Gpts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "clocks": clocks, "gpu_launches": 0}
        print(json.dumps(line), flush=True)
        return
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_rate(cfgd, models, shot, threads, 1, 2)
    r0, _ = cpu_rate(cfgd, models, shot, threads, 2, 6)
    per_step = updated_cells(cfgd) / (r0 * 1e9)
    nsteps = max(4, min(2000, int(6.0 / per_step)))  # ~6 s of CPU work per bench step
    rates, secs = [], 0.0
    for _ in range(args.steps):
        r, info = cpu_rate(cfgd, models, shot, threads, 2, 2 + nsteps)
        rates.append(r)
        secs += info["seconds"]
    value = float(np.mean(rates))
    sample = (f"{cfgd['physics']} {meta['model']} grid, {nsteps} time steps per bench step "
              f"(difference of two oracle runs, literal arithmetic)")
    line = {"metric": "Gpts/s", "value": value, "unit": "Gpts/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * secs / max(args.steps, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": config, "impl": "reference",
            "reference_kind": "cpu port (reference kernels not built here)",
            "cpu_baseline": {"value": value, "unit": "Gpts/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "Gpts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0}
    print(json.dumps(line), flush=True)


def tti_windows(nt_override=None):
    """The TTI survey of uneven apertures: 512 x 512 x 320 model, d 12.5 m, nt 3000;
    smooth seeded fields (v 1500-5000 seed 7, epsilon 0-0.3 seed 8, delta <= epsilon
    in 0-0.15 seed 9, tilt 0-45 deg seed 10, azimuth 0-360 deg seed 11, radians);
    48 windows with sizes uniform per axis in [160, 320] and placements uniform
    inside the model (seed 12), each with its own 20-cell PML and a 15 Hz Ricker at
    its centre, depth 2."""
    import synthetic as S
    nx, ny, nz, d, vmax = 512, 512, 320, 12.5, 5000.0
    models = S.tti_model(nx, ny, nz, vmax)
    wins, shots = S.tti_windows(nx, ny, nz)
    dt = np.float32(0.4 * d / (vmax * np.sqrt(1.6)))
    nt = nt_override or 3000
    cfg = dict(physics="tti", nx=nx, ny=ny, nz=nz, dx=d, dy=d, dz=d, nt=nt, dt=float(dt), fm=15.0, npml=20)
    return cfg, models, wins, shots


def run_windows(args):
    """Bench step = one a3d_run_batch call over --windows apertures (graph replay on)."""
    import a3d
    import build as pkg_build
    pkg_build.build()
    cfgd, models, wins, shots = tti_windows(args.nt or None)
    k = max(1, min(args.windows, len(wins)))
    cfg = a3d.make_config("tti", cfgd["nx"], cfgd["ny"], cfgd["nz"], dx=cfgd["dx"], dy=cfgd["dy"], dz=cfgd["dz"],
                          nt=cfgd["nt"], dt=cfgd["dt"], fm=cfgd["fm"], npml=cfgd["npml"])
    nt = cfgd["nt"]
    cells = sum((w[3] + 2 * 20 - 8) * (w[4] + 2 * 20 - 8) * (w[5] + 2 * 20 - 8) for w in wins[:k])
    for _ in range(args.warmup):
        a3d.run_batch(cfg, models, shots[:1], windows=wins[:1], graph=True)
    dev_ms, wall = 0.0, 0.0
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            _, ms = a3d.run_batch(cfg, models, shots[:k], windows=wins[:k], graph=True)
            wall += time.perf_counter() - t0
            dev_ms += sum(ms)
    value = cells * nt * args.steps / (dev_ms / 1000.0) / 1e9
    line = {"metric": "Gpts/s", "value": value, "unit": "Gpts/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "tti1order_512x512x320_windows_nt%d" % nt, "windows": k,
                       "window_sizes": [list(w[3:]) for w in wins[:k]], "npml": 20, "storage": "fp32",
                       "graph": True},
            "shots_per_hour": 3600.0 * k * args.steps / wall,
            "e2e": {"value": cells * nt * args.steps / wall / 1e9, "unit": "Gpts/s",
                    "call": "a3d_run_batch (host model, per-window crop, upload, loop, record download)"},
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def run_vti_batch(args):
    """VTI survey of the 384 x 384 x 256 model (the vti384 workload) in multi-shot
    sweeps: a bench step is one launch sequence advancing --batch shots of the 8 x 8
    surface shot grid (x, y in 24 + 48 i, depth 2) through all nt = 2500 steps.
    value = updated cells x nt x shots / device time; beside it the same model's
    single-shot FP32 path (one shot per run, as the reference runs them), the
    shots/hour of both and their ratio, and the record error against FP64 of the
    sweep's first shot and of the single FP32 shot."""
    import a3d
    import build as pkg_build
    import synthetic as S
    pkg_build.build()
    cfgd, models, _, meta = workload("vti384", args.nt or None)
    K = max(1, args.batch)
    shots = S.vti_shot_grid()[:K]
    if args.scale > 1:  # a smaller case of the same workload (profiling): every axis / scale
        f = args.scale
        cfgd = dict(cfgd, nx=cfgd["nx"] // f, ny=cfgd["ny"] // f, nz=cfgd["nz"] // f)
        models = S.vti_model(cfgd["nx"], cfgd["ny"], cfgd["nz"], 4500.0)
        shots = S.vti_shot_grid(first=24 // f, step=48 // f)[:K]
        meta = dict(meta, model="%dx%dx%d" % (cfgd["nx"], cfgd["ny"], cfgd["nz"]))
    nt = cfgd["nt"]
    cells = updated_cells(cfgd)

    def cfg_of(storage, batch=0):
        return a3d.make_config("vti", cfgd["nx"], cfgd["ny"], cfgd["nz"], dx=cfgd["dx"], dy=cfgd["dy"],
                               dz=cfgd["dz"], nt=nt, dt=cfgd["dt"], fm=cfgd["fm"], npml=cfgd["npml"],
                               storage=storage, batch=batch)
    # the single-shot FP32 path on the same model and first shot
    e1 = a3d.Engine(cfg_of(a3d.FP32), models)
    e1.run_device(*shots[0])
    single_ms = e1.run_device(*shots[0])
    rec32 = e1.run(*shots[0]) if not args.no_fp64 else None
    e1.close()
    # the multi-shot sweeps
    eb = a3d.Engine(cfg_of(STORAGE[args.storage], K), models)
    for _ in range(args.warmup):
        eb.run_shots(shots, to_host=False)
    eb.set_profiling(True)
    dev_ms = 0.0
    with ClockSampler(0) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            dev_ms += eb.run_shots(shots, with_time=True, to_host=False)[1]
        wall = time.perf_counter() - t0
    kms, kn = eb.kernel_times()
    desc = eb.describe()
    rec_b = eb.record(0) if not args.no_fp64 else None
    dev_bytes = eb.device_bytes()
    eb.close()
    err = {}
    if not args.no_fp64:
        e64 = a3d.Engine(cfg_of(a3d.FP64), models)
        rec64 = e64.run(*shots[0]).astype(np.float64)
        e64.close()
        n64 = np.linalg.norm(rec64.ravel())
        err = {"sweep_shot0": float(np.linalg.norm((rec_b - rec64).ravel()) / n64),
               "single_fp32_shot0": float(np.linalg.norm((rec32 - rec64).ravel()) / n64)}
    ms_step = dev_ms / args.steps
    value = cells * nt * K * args.steps / (dev_ms / 1000.0) / 1e9
    sph = 3600.0 * 1000.0 * K / ms_step
    sph1 = 3600.0 * 1000.0 / single_ms
    peak, peak_kind = measured_peak()
    es = 4 if args.storage == "fp32" else 2
    # compulsory bytes per cell and shot: wavefields read and written per shot, the
    # model parameters once per tile for the whole sweep (1/rho in the velocity
    # sweep; rho, vp, epsilon, delta in the stress sweep); velocity sweep: P, Q, u, v,
    # w read, u, v, w written; stress sweep: u, v, w, P, Q read, P, Q written
    ep = 4 if args.storage == "fp16v" else es  # bytes of P, Q
    kb = (es * 6 + ep * 2 + 4.0 / K, es * 3 + ep * 4 + 16.0 / K)
    per = [kms[i] / kn[i] if kn[i] else 0.0 for i in range(2)]
    dom = 0 if per[0] >= per[1] else 1
    achieved = kb[dom] * cells * K / (per[dom] / 1000.0) / 1e9
    line = {"metric": "Gpts/s", "value": value, "unit": "Gpts/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if es == 4 else (
                "f32 arithmetic, f16 u, v, w, f32 P, Q" if args.storage == "fp16v" else
                f"f32 arithmetic, {args.storage} wavefields"),
            "data": "synthetic",
            "config": dict(meta, workload="vti1order_%s_nt%d_sweep%d" % (meta["model"], nt, K),
                           shots=[list(x) for x in shots], batch=K, storage=args.storage, parallelism="replicas1",
                           l2="inputs larger than L2: %d MB of wavefields and model per shot" %
                              (dev_bytes // K // 2**20)),
            "shots_per_hour": sph, "single_shot_fp32": {"ms_per_shot": single_ms, "shots_per_hour": sph1},
            "shots_per_hour_ratio": sph / sph1, "rel_l2_vs_fp64": err,
            "roofline": {"bound": "hbm", "kernel": ("vti_vel", "vti_stress")[dom], "achieved": achieved,
                         "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": None,
                         "peak_source": peak_kind, "bytes_per_cell_and_shot": kb[dom],
                         "kernel_ms_per_launch": per[dom]},
            "device_bytes": dev_bytes, "wall_s_timed": wall, "clocks": clk.summary(),
            "tuning": desc.get("kernels"), "gpu_launches": int(kn[0] + kn[1])}
    print(json.dumps(line), flush=True)


def round_params(models, kind):
    """Model arrays rounded to float16 or bfloat16 (round to nearest even), as float32."""
    out = {}
    for k, v in models.items():
        a = np.ascontiguousarray(v, np.float32)
        if kind == "fp16":
            out[k] = a.astype(np.float16).astype(np.float32)
        else:
            b = a.view(np.uint32).astype(np.uint64)
            out[k] = ((b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000).astype(np.uint32).view(np.float32)
    return out


def run_param_rounding(args):
    """Record error from 16-bit model parameters: the FP64 engine on the workload's
    models rounded to float16 / bfloat16 against the FP64 engine on the exact models
    (no timing; one JSON line per format)."""
    import a3d
    import build as pkg_build
    pkg_build.build()
    cfgd, models, shot, meta = workload(args.workload, args.nt or None)

    def rec(m):
        cfg = a3d.make_config(cfgd["physics"], cfgd["nx"], cfgd["ny"], cfgd["nz"], dx=cfgd["dx"], dy=cfgd["dy"],
                              dz=cfgd["dz"], nt=cfgd["nt"], dt=cfgd["dt"], fm=cfgd["fm"], npml=cfgd["npml"],
                              rec_z=cfgd.get("rec_z", -1), storage=a3d.FP64)
        e = a3d.Engine(cfg, m)
        try:
            return e.run(*shot).astype(np.float64)
        finally:
            e.close()

    r64 = rec(models)
    n64 = np.linalg.norm(r64.ravel())
    for kind in ("fp16", "bf16"):
        r = rec(round_params(models, kind))
        print(json.dumps({"workload": meta["workload"], "params": kind, "engine": "fp64",
                          "rel_l2_vs_exact_params": float(np.linalg.norm((r - r64).ravel()) / n64)}), flush=True)


def run_learned(args):
    """The learned absorbing rim against the PML (isotropic 256^3, d 10 m, nt 2000,
    20 Hz Ricker at the centre, depth 8): a bench step is one learned-rim shot
    (value = updated cells of its padded grid x nt / device time); beside it one
    shot each of the 20-cell PML, the 10-cell PML (the rim's own padding) and the
    60-cell-PML judge, with device time, device memory and the reflection energy
    ratios against the judge (record over all samples; model-interior pressure at
    every 250th step)."""
    import a3d
    import build as pkg_build
    import learned_abc as L
    import synthetic as S
    pkg_build.build()
    n, dx, vmax = 256, 10.0, 4500.0
    md = S.iso_model(n, 2, vmax)
    dt = S.cfl_dt(dx, vmax)
    nt = args.nt or 2000
    shot = (n // 2, n // 2, 8)
    params = L.load_params(args.params or L.PARAMS_FILE)
    cfg = a3d.make_config("iso", n, n, n, dx, dx, dx, nt=nt, dt=dt, fm=20.0, npml=a3d.CLOSURE_PAD,
                          boundary="learned")
    e = a3d.Engine(cfg, md)
    e.set_closure(params)
    for _ in range(args.warmup):
        e.run_device(*shot)
    dev_ms = 0.0
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            dev_ms += e.run_device(*shot)
    e.set_profiling(True)
    e.run_device(*shot)
    kms, kn = e.kernel_times()
    cms, cn = e.closure_times()
    e.close()
    cells = (n + 2 * a3d.CLOSURE_PAD - 8) ** 3
    ms = dev_ms / args.steps
    ratios = L.reflection(md["vel"], md["rho"], shot, nt, dt, params)
    ratios["choice"] = L.choose_boundary(ratios)
    line = {"metric": "Gpts/s", "value": cells * nt / (ms / 1000.0) / 1e9, "unit": "Gpts/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (closure bf16 operands, f32 accumulation)",
            "data": "synthetic",
            "config": {"workload": "iso1order_256cube_learned_rim_nt%d" % nt, "rim_cells": 6,
                       "closure": "3x3x3 conv 8->32 relu, 3x3x3 conv 32->4 per face, %d parameters"
                                  % a3d.CLOSURE_NPARAM, "l2": "inputs larger than L2"},
            "model_interior_gpts": n ** 3 * nt / (ms / 1000.0) / 1e9,
            "per_step_ms": {"velocity": kms[0] / max(kn[0], 1), "stress": kms[1] / max(kn[1], 1),
                            "closure": cms / max(cn, 1)},
            "comparison": ratios, "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="iso256",
                    choices=["iso256", "2o128", "2o128lit", "vti384", "vti384batch", "tti256", "ttiwin",
                             "learned"])
    ap.add_argument("--batch", type=int, default=32, help="vti384batch: shots per multi-shot sweep")
    ap.add_argument("--scale", type=int, default=1, help="vti384batch: divide every model axis (profiling cases)")
    ap.add_argument("--params", default="", help="learned: closure weights (.npy; default the package's)")
    ap.add_argument("--windows", type=int, default=4, help="ttiwin: apertures per bench step (of 48)")
    ap.add_argument("--nt", type=int, default=0, help="override nt (profiling runs only)")
    ap.add_argument("--tile-x", type=int, default=0)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 error check")
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--no-legacy", action="store_true", help="skip the drop-in entry point's end-to-end timing")
    ap.add_argument("--param-rounding", action="store_true",
                    help="no timing: record error of 16-bit model parameters (FP64 engine)")
    ap.add_argument("--storage", default="fp32", choices=list(STORAGE),
                    help="wavefield storage (bf16 / fp16: isotropic and VTI engines; arithmetic stays fp32)")
    args = ap.parse_args()
    # three warm-up steps at least for the shot workloads; a multi-shot sweep of the
    # batched survey is itself 30-120 s of device time, after the autotuner has run
    # every kernel, so one warm-up sweep is allowed there
    if args.impl == "ours" and args.workload != "vti384batch":
        args.warmup = max(args.warmup, 3)

    if args.workload == "ttiwin":
        run_windows(args)
        return
    if args.workload == "learned":
        run_learned(args)
        return
    if args.workload == "vti384batch":
        run_vti_batch(args)
        return
    if args.param_rounding:
        run_param_rounding(args)
        return
    cfgd, models, shot, meta = workload(args.workload, args.nt or None)
    meta["storage"] = args.storage
    if args.storage != "fp32" and cfgd["physics"] not in ("iso", "vti", "tti"):
        raise SystemExit("2-byte storage is built for the 1st-order engines only")
    if args.storage == "fp16v" and cfgd["physics"] not in ("vti", "tti"):
        raise SystemExit("fp16v storage is built for the VTI and TTI engines only")
    if args.impl == "reference":
        run_reference(args, cfgd, models, shot, meta)
        return

    import a3d
    import build as pkg_build
    pkg_build.build()
    ws, rank, local = dist_env()
    dev = local
    group = None
    if ws > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(dev)
        dist.init_process_group("nccl")
        group = dist
    eng = cfgd["physics"]
    cfg = a3d.make_config(eng, cfgd["nx"], cfgd["ny"], cfgd["nz"], dx=cfgd["dx"], dy=cfgd["dy"],
                          dz=cfgd["dz"], nt=cfgd["nt"], dt=cfgd["dt"], fm=cfgd["fm"], npml=cfgd["npml"],
                          rec_z=cfgd.get("rec_z", -1), mute=cfgd.get("mute", False), tile_x=args.tile_x,
                          storage=STORAGE[args.storage])
    e = a3d.Engine(cfg, models, device=dev)
    snap_every = cfgd.get("snap_every", 0)

    def shot_device(sx_):
        """one shot, inputs resident; device ms of its time loop (snapshots, when the
        workload takes them, cropped on the device and copied out while it runs)"""
        if snap_every:
            return e.run(sx_, shot[1], shot[2], snap_every=snap_every, with_time=True)[-1]
        return e.run_device(sx_, shot[1], shot[2])
    # replicas: the job's shots run along x, one per rank, split round-robin as
    # the reference splits shots over nodes
    import a3d_dist
    job_shots = [(min(cfgd["nx"] - 1, shot[0] + 4 * k), shot[1], shot[2]) for k in range(ws)]
    sx = a3d_dist.shots_for_rank(job_shots, rank, ws)[0][0]
    for _ in range(args.warmup):
        shot_device(sx)

    def barrier():
        if group:
            import torch
            torch.cuda.synchronize(dev)
            group.barrier()

    # ---- timed region: K shots, inputs resident
    barrier()
    if not snap_every:
        e.set_profiling(True)
    dev_ms = 0.0
    with ClockSampler(dev) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            dev_ms += shot_device(sx)
        wall = time.perf_counter() - t0
    barrier()
    if snap_every:  # kernel events separately, on one shot without snapshots
        e.set_profiling(True)
        e.run_device(sx, shot[1], shot[2])
    kms, kn = e.kernel_times()
    e.set_profiling(False)
    desc = e.describe()
    tuning = desc["kernels"][:1] if desc.get("fused") else desc["kernels"]
    dev_ms = a3d_dist.max_over_ranks(dev_ms, group, f"cuda:{dev}" if group else None)
    cells = updated_cells(cfgd)
    nt = cfgd["nt"]
    value = cells * nt * args.steps * ws / (dev_ms / 1000.0) / 1e9
    ms_per_step = dev_ms / args.steps

    # ---- roofline of the dominant kernel
    peak, peak_kind = measured_peak()
    two = args.storage != "fp32"
    mixed = args.storage == "fp16v"
    kb = (KERNEL_BYTES_MIXED if mixed else KERNEL_BYTES_2B if two else KERNEL_BYTES)[eng]
    if desc.get("fused"):  # one fused step per time step: u, v, w, P, 1/rho, rho, vp read, u, v, w, P written
        kb = (FUSED_BYTES, None)
    step_b = (STEP_BYTES_MIXED if mixed else STEP_BYTES_2B if two else STEP_BYTES)[eng]
    per = [kms[i] / kn[i] if kn[i] else 0.0 for i in range(2)]
    dom = 0 if (per[0] >= per[1] or kb[1] is None) else 1
    achieved = kb[dom] * cells / (per[dom] / 1000.0) / 1e9
    step_gbs = step_b * cells * nt * args.steps / (dev_ms / 1000.0) / 1e9
    kname = {("iso", 0): "iso_vel", ("iso", 1): "iso_stress", ("2o", 0): "k2o_step", ("vti", 0): "vti_vel",
             ("vti", 1): "vti_stress", ("tti", 0): "tti_vel", ("tti", 1): "tti_stress"}.get((eng, dom), "?")
    if desc.get("fused"):
        kname = "iso_step"
    tr = traffic_per_launch(meta["workload"] + ("" if args.storage == "fp32" else "_" + args.storage))
    # DRAM bytes of the launch shape the tuner picked ("kernel@<tile x>x<rows>"), else
    # of the kernel's profiled shape
    kd = tuning[min(dom, len(tuning) - 1)] if tuning else {}
    shape_key = "%s@%dx%d" % (kname, kd.get("tile_x", 0), kd.get("rows", 0))
    traffic = (tr.get(shape_key, tr.get(kname)) if isinstance(tr, dict) else None)
    roofline = {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic,
                "peak_source": peak_kind, "bytes_per_cell": kb[dom],
                "kernel_ms_per_launch": per[dom],
                "step": {"bytes_per_cell": step_b, "achieved": step_gbs, "frac": step_gbs / peak}}
    if traffic and per[dom] > 0:
        # the DRAM bytes ncu measured for one launch of this kernel over this run's
        # event-timed launch: how fast the kernel actually draws from HBM, PML split
        # components and halo re-reads included
        roofline["traffic_gbs"] = traffic / (per[dom] / 1000.0) / 1e9
        roofline["traffic_frac"] = roofline["traffic_gbs"] / peak

    # ---- FP64 error of the FP32 record (outside the timed region)
    rel = None
    if not args.no_fp64 and rank == 0:
        rec32 = e.run(sx, shot[1], shot[2])
        cfg64 = a3d.make_config(eng, cfgd["nx"], cfgd["ny"], cfgd["nz"], dx=cfgd["dx"], dy=cfgd["dy"],
                                dz=cfgd["dz"], nt=cfgd["nt"], dt=cfgd["dt"], fm=cfgd["fm"], npml=cfgd["npml"],
                                rec_z=cfgd.get("rec_z", -1), mute=cfgd.get("mute", False), storage=a3d.FP64)
        e64 = a3d.Engine(cfg64, models, device=dev)
        rec64 = e64.run(sx, shot[1], shot[2])
        e64.close()
        d = np.linalg.norm((rec32.astype(np.float64) - rec64).ravel())
        rel = float(d / np.linalg.norm(rec64.astype(np.float64).ravel()))
    e.close()

    # ---- e2e through the host-buffer C-ABI call (H2D model, loop, D2H record)
    # model arrays copied to the device per call, unpadded (padding runs on the device):
    # 2O v; ISO v, rho; VTI v, rho, epsilon, delta; TTI v, epsilon, delta and the host's
    # cos / sin of tilt and azimuth
    n_upload = {"2o": 1, "iso": 2, "vti": 4, "tti": 7}[eng]
    h2d = 4 * cfgd["nx"] * cfgd["ny"] * cfgd["nz"] * n_upload
    d2h = 4 * cfgd["nx"] * cfgd["ny"] * cfgd["nt"]
    e2e_val = None
    if snap_every:  # snapshots come back as host arrays: one window per snapshot
        d2h += 4 * cfgd["nx"] * cfgd["ny"] * cfgd["nz"] * len(range(0, cfgd["nt"], snap_every))

    def e2e_once():
        if not snap_every:
            a3d.forward_host(cfg, models, [(sx, shot[1], shot[2])], device=dev)
            return
        eh = a3d.Engine(cfg, models, device=dev)  # model upload and set-up
        try:
            eh.run(sx, shot[1], shot[2], snap_every=snap_every)
        finally:
            eh.close()

    if args.e2e_steps > 0:
        e2e_once()  # warm
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            e2e_once()
        e2e_s = time.perf_counter() - t0
        barrier()
        e2e_val = cells * nt * args.e2e_steps * ws / e2e_s / 1e9

    # ---- the drop-in entry point end to end (model files in, record file out)
    legacy = None
    if rank == 0 and args.storage == "fp32" and not args.no_legacy:
        legacy = legacy_e2e(cfgd, models, (sx, shot[1], shot[2]), dev)

    # ---- CPU baseline (rank 0, N = 1 only)
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        r, info = cpu_rate(cfgd, models, shot, threads)
        cpu = {"value": r, "unit": "Gpts/s", "cores": threads, "kind": "port",
               "sample": f"{meta['model']} grid, {info['steps']} time steps (difference of two oracle "
                         f"runs, literal arithmetic), {info['seconds']:.1f} s"}

    if rank == 0:
        clocks = clk.summary()
        line = {"metric": "Gpts/s", "value": value, "unit": "Gpts/s", "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": {"fp32": "f32", "fp16v": "f32 arithmetic, f16 u, v, w, f32 P, Q"}.get(
                    args.storage, f"f32 arithmetic, {args.storage} wavefields"), "data": "synthetic",
                "config": bench_config(meta, cfgd, ws),
                "shots_per_hour": 3600.0 * 1000.0 / ms_per_step * ws,
                "rel_l2_vs_fp64": rel,
                "roofline": roofline, "cpu_baseline": cpu,
                "e2e": {"value": e2e_val, "unit": "Gpts/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                        "call": "a3d_engine_create + a3d_engine_run (record and snapshots to host) + destroy"
                        if snap_every else "a3d_forward_host", "legacy_entry_point": legacy},
                "wall_s_timed": wall, "clocks": clocks,
                "tuning": {"fused_step": bool(desc.get("fused")), "tile_x_request": args.tile_x,
                           "kernels": tuning},
                # our kernels in the timed region: the step kernels, plus one crop per
                # snapshot when the workload takes snapshots
                "gpu_launches": int(kn[0] + kn[1]) if not snap_every else
                args.steps * (nt + len(range(0, nt, snap_every)))}
        print(json.dumps(line), flush=True)
    if group:
        group.destroy_process_group()


if __name__ == "__main__":
    main()
