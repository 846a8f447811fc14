"""Learned absorbing rim for the isotropic engine.

The reference absorbs outgoing waves with a 20-cell split PML on every face
(..iso..:263-291).  The learned rim replaces it by 6 undamped cells whose state a
small network corrects after every step (the kernels and the exact formula are in
csrc/a3d_closure.h).  This module makes and uses it:

* teacher data: wide-PML runs (40 cells) on seeded smooth models, tapped at
  consecutive steps and cropped to the rim grid (`teacher_set`);
* training on the GPU with the library's own kernels (`train`, `a3d.Closure`);
* the judge: reflection energy of a run against a much wider PML (60 cells) on the
  same model, shot and time axis (`reflection`), over the model interior;
* the fallback: `choose_boundary` keeps the learned rim only where its reflection
  is below the 20-cell PML's on a held-out model, otherwise the PML.

Command line (runs on a GPU):
    python acoustic3d-fd_gb300/learned_abc.py train --models 200 --n 64 --out rim.npy
    python acoustic3d-fd_gb300/learned_abc.py judge --params rim.npy --n 96
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import a3d  # noqa: E402
import synthetic as S  # noqa: E402

PARAMS_FILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "rim_closure.npy")
NW1, NW2, NG = 32 * 8 * 27, 6 * 4 * 32 * 27, 6 * 6 * 4


def smooth_velocity(nx, ny, nz, seed, lo=1500.0, hi=4500.0, sigma=8.0):
    """Seeded smooth velocity (shape (ny, nx, nz)), the generator of synthetic.py."""
    return S.smooth_field3(nx, ny, nz, seed, lo, hi, sigma)


gardner = S.gardner


def init_params(seed=0):
    """He-initialised W1, small W2 (the rim starts close to undamped), gains 1."""
    rng = np.random.default_rng(seed)
    w1 = rng.normal(0.0, np.sqrt(2.0 / (8 * 27)), NW1)
    w2 = rng.normal(0.0, 0.1 / np.sqrt(32 * 27), NW2)
    g = np.ones(NG)
    return np.concatenate([w1, w2, g]).astype(np.float32)


def split_params(p):
    p = np.asarray(p, np.float32)
    return (p[:NW1].reshape(32, 8, 3, 3, 3), p[NW1:NW1 + NW2].reshape(6, 4, 32, 3, 3, 3),
            p[NW1 + NW2:].reshape(6, 6, 4))


TAPS = (100, 160, 220, 300, 400, 550)


def _shot(n, seed0, m):
    rng = np.random.default_rng(seed0 + m + 100000)
    return tuple(int(v) for v in rng.integers(n // 4, 3 * n // 4, 3))


def teacher_set(cl: a3d.Closure, n, n_models, seed0=1000, taps=TAPS, wide=40, dx=10.0, fm=20.0, vmax=4500.0,
                device=0, log=None):
    """Add len(taps) teacher pairs per model to the closure's sample set.

    Model m (closure model id m): smooth velocity (seed seed0 + m, 1500..vmax m/s),
    Gardner density, a 20 Hz Ricker at a seeded position in the middle half of the
    model, dt from CFL 0.4; the run has a `wide`-cell PML and is tapped at t and
    t + 1 for every t in taps, cropped to the rim grid (model + 10 cells per face)."""
    dt = S.cfl_dt(dx, vmax)
    steps = [s for t in taps for s in (t, t + 1)]
    fb = cl.state_floats() * 4
    for m in range(n_models):
        md = S.rim_training_model(n, seed0 + m, vmax)
        cfg = a3d.make_config("iso", n, n, n, dx, dx, dx, nt=max(taps) + 2, dt=dt, fm=fm, npml=wide, tile_x=16)
        e = a3d.Engine(cfg, md, device)
        try:
            buf = cl.staging(len(steps))
            e.set_tap(steps, wide - a3d.CLOSURE_PAD, buf)
            e.run_device(*_shot(n, seed0, m))
        finally:
            e.close()
        mid = cl.add_model(md["vel"], md["rho"], dx, dx, dx, dt)
        assert mid == m
        for k in range(len(taps)):
            cl.add_sample(mid, buf + 2 * k * fb, buf + (2 * k + 1) * fb)
        if log and (m + 1) % 50 == 0:
            log(f"teacher models {m + 1}/{n_models}, samples {cl.num_samples()}")
    return dt


def student_set(cl: a3d.Closure, params, n, models, seed0=1000, taps=TAPS, wide=40, dx=10.0, fm=20.0,
                vmax=4500.0, device=0):
    """On-policy pairs: the learned-rim engine's own state at t (closed loop with the
    current weights) with the wide-PML teacher's state at t + 1, for the listed
    model ids (added by teacher_set).  States that ran away are refused.
    Returns (pairs added, pairs refused)."""
    dt = S.cfl_dt(dx, vmax)
    fb = cl.state_floats() * 4
    added = refused = 0
    for m in models:
        md = S.rim_training_model(n, seed0 + m, vmax)
        shot = _shot(n, seed0, m)
        buf = cl.staging(2 * len(taps))
        cs = a3d.make_config("iso", n, n, n, dx, dx, dx, nt=max(taps) + 2, dt=dt, fm=fm, npml=a3d.CLOSURE_PAD,
                             boundary="learned", tile_x=16)
        cw = a3d.make_config("iso", n, n, n, dx, dx, dx, nt=max(taps) + 2, dt=dt, fm=fm, npml=wide, tile_x=16)
        for cfg, steps, off, dst in ((cs, list(taps), 0, buf), (cw, [t + 1 for t in taps], wide - a3d.CLOSURE_PAD,
                                                                 buf + len(taps) * fb)):
            e = a3d.Engine(cfg, md, device)
            try:
                if cfg.boundary:
                    e.set_closure(params)
                e.set_tap(steps, off, dst)
                e.run_device(*shot)
            finally:
                e.close()
        for k in range(len(taps)):
            try:
                cl.add_sample(m, buf + k * fb, buf + (len(taps) + k) * fb)
                added += 1
            except a3d.A3DError:
                refused += 1
    return added, refused


def train(n=64, n_models=200, seed0=1000, epochs=12, batch=8, lr=1e-3, seed=0, device=0, log=print, rounds=3,
          round_models=40, round_epochs=6, decay=1e-4, monitor=None):
    """Teacher data and Adam, then `rounds` rounds that add on-policy pairs of
    round_models models (the closure's own closed-loop states, teacher targets) and
    train on everything gathered.  monitor(params) -> dict is logged after each
    stage.  Returns (params, loss per epoch, info)."""
    t0 = time.time()
    cl = a3d.Closure(n, n, n, device)
    info = {"stages": []}
    try:
        teacher_set(cl, n, n_models, seed0, device=device, log=log)
        info["teacher_s"] = time.time() - t0
        cl.set_params(init_params(seed))
        cl.set_decay(decay)
        losses = [float(x) for x in cl.train(epochs, batch, lr, seed)]
        stage = {"samples": cl.num_samples(), "loss": losses[-1]}
        if monitor:
            stage["monitor"] = monitor(cl.params())
        info["stages"].append(stage)
        log(json.dumps(stage))
        best = (stage.get("monitor", {}).get("learned", 0.0), cl.params())
        for r in range(rounds):
            ids = [(r * round_models + k) % n_models for k in range(round_models)]
            added, refused = student_set(cl, cl.params(), n, ids, seed0, device=device)
            rl = [float(x) for x in cl.train(round_epochs, batch, lr * 0.7 ** (r + 1), seed + r + 1)]
            losses += rl
            stage = {"round": r, "added": added, "refused": refused, "samples": cl.num_samples(), "loss": rl[-1]}
            if monitor:
                stage["monitor"] = monitor(cl.params())
                if stage["monitor"]["learned"] < best[0]:
                    best = (stage["monitor"]["learned"], cl.params())
            info["stages"].append(stage)
            log(json.dumps(stage))
        info["total_s"] = time.time() - t0
        info["samples"] = cl.num_samples()
        # with a monitor, the weights of the stage that reflected least
        return (best[1] if monitor else cl.params()), losses, info
    finally:
        cl.close()


def run_shot(vel, rho, shot, nt, dt, dx=10.0, fm=20.0, boundary="pml", npml=20, params=None, snap_every=0,
             device=0, tile_x=0):
    """One isotropic shot; returns (record, snapshots or None, device ms, device bytes)."""
    ny, nx, nz = vel.shape
    if boundary == "learned":
        cfg = a3d.make_config("iso", nx, ny, nz, dx, dx, dx, nt=nt, dt=dt, fm=fm, npml=a3d.CLOSURE_PAD,
                              boundary="learned", tile_x=tile_x)
    else:
        cfg = a3d.make_config("iso", nx, ny, nz, dx, dx, dx, nt=nt, dt=dt, fm=fm, npml=npml, tile_x=tile_x)
    e = a3d.Engine(cfg, {"vel": vel, "rho": rho}, device)
    try:
        if boundary == "learned":
            e.set_closure(params)
        out = e.run(*shot, snap_every=snap_every, snap_skip0=True, with_time=True)
        bytes_ = e.device_bytes()
    finally:
        e.close()
    if snap_every:
        rec, snaps, ms = out
    else:
        (rec, ms), snaps = out, None
    return rec, snaps, ms, bytes_


def reflection(vel, rho, shot, nt, dt, params=None, judge=60, pml=20, snap_every=250, dx=10.0, fm=20.0,
               device=0):
    """Reflection energy ratios against a judge run with a `judge`-cell PML:

    record: |rec - rec_judge|^2 / |rec_judge|^2 over all receivers and samples;
    volume: the same for the model-interior pressure, summed over the snapshots
    taken every snap_every steps.  Returns {"judge": {...}, "pml": {...} (pml cells),
    "pml_thin": {...} (the learned rim's 10-cell padding as a PML), "learned": {...}}."""
    out = {}
    rj, sj, msj, bj = run_shot(vel, rho, shot, nt, dt, dx, fm, "pml", judge, snap_every=snap_every, device=device)
    ej_r, ej_v = float(np.sum(rj.astype(np.float64) ** 2)), float(np.sum(sj.astype(np.float64) ** 2))
    out["judge"] = {"npml": judge, "ms": msj, "device_bytes": bj}
    runs = [("pml", "pml", pml), ("pml_thin", "pml", a3d.CLOSURE_PAD)]
    if params is not None:
        runs.append(("learned", "learned", None))
    for name, b, w in runs:
        r, s, ms, by = run_shot(vel, rho, shot, nt, dt, dx, fm, b, w or 20, params, snap_every, device)
        ok = bool(np.all(np.isfinite(r)) and np.all(np.isfinite(s)))
        out[name] = {"ms": ms, "device_bytes": by, "finite": ok,
                     "record_ratio": float(np.sum((r.astype(np.float64) - rj) ** 2) / ej_r) if ok else float("inf"),
                     "volume_ratio": float(np.sum((s.astype(np.float64) - sj) ** 2) / ej_v) if ok else float("inf")}
    return out


def choose_boundary(ratios: dict) -> str:
    """'learned' when the learned rim reflects less than the PML on the judged run
    (both ratios finite and lower), else 'pml' — the PML is the fallback."""
    lr, pm = ratios.get("learned"), ratios["pml"]
    if lr and lr["finite"] and lr["record_ratio"] < pm["record_ratio"] and lr["volume_ratio"] < pm["volume_ratio"]:
        return "learned"
    return "pml"


def load_params(path=PARAMS_FILE):
    p = np.load(path).astype(np.float32)
    if p.size != a3d.CLOSURE_NPARAM:
        raise ValueError(f"{path}: {p.size} parameters, expected {a3d.CLOSURE_NPARAM}")
    return p


def _main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--models", type=int, default=200)
    t.add_argument("--n", type=int, default=64)
    t.add_argument("--epochs", type=int, default=12)
    t.add_argument("--batch", type=int, default=8)
    t.add_argument("--lr", type=float, default=1e-3)
    t.add_argument("--out", default=PARAMS_FILE)
    t.add_argument("--rounds", type=int, default=3)
    t.add_argument("--round-models", type=int, default=40)
    t.add_argument("--round-epochs", type=int, default=6)
    t.add_argument("--decay", type=float, default=1e-4)
    t.add_argument("--monitor-n", type=int, default=0)
    t.add_argument("--monitor-nt", type=int, default=800)
    j = sub.add_parser("judge")
    j.add_argument("--params", default=PARAMS_FILE)
    j.add_argument("--n", type=int, default=96)
    j.add_argument("--nt", type=int, default=1200)
    j.add_argument("--seed", type=int, default=1999)
    r = sub.add_parser("run", help="one learned-rim shot on a seeded model (timing, profiling)")
    r.add_argument("--params", default=PARAMS_FILE)
    r.add_argument("--n", type=int, default=96)
    r.add_argument("--nt", type=int, default=20)
    r.add_argument("--seed", type=int, default=3)
    a = ap.parse_args(argv)
    if a.cmd == "run":
        md = S.iso_model(a.n, a.seed)
        cfg = a3d.make_config("iso", a.n, a.n, a.n, 10.0, 10.0, 10.0, nt=a.nt, dt=S.cfl_dt(10.0, 4500.0), fm=20.0,
                              npml=a3d.CLOSURE_PAD, boundary="learned", tile_x=16)
        e = a3d.Engine(cfg, md)
        e.set_closure(load_params(a.params))
        _, ms = e.run(a.n // 2, a.n // 2, 8, with_time=True)
        e.close()
        print(json.dumps({"n": a.n, "nt": a.nt, "ms": ms}))
        return
    if a.cmd == "train":
        mon = None
        if a.monitor_n:
            md = S.rim_training_model(a.monitor_n, 1999)
            c = a.monitor_n // 2
            dt = S.cfl_dt(10.0, 4500.0)

            def mon(p):
                r = reflection(md["vel"], md["rho"], (c, c, 8), a.monitor_nt, dt, p)
                return {k: r[k].get("record_ratio") for k in ("pml", "pml_thin", "learned")}
        p, losses, info = train(a.n, a.models, epochs=a.epochs, batch=a.batch, lr=a.lr, rounds=a.rounds,
                                round_models=a.round_models, round_epochs=a.round_epochs, decay=a.decay,
                                monitor=mon, log=lambda s: print(s, file=sys.stderr, flush=True))
        os.makedirs(os.path.dirname(os.path.abspath(a.out)), exist_ok=True)
        np.save(a.out, p)
        print(json.dumps({"losses": [float(x) for x in losses], **info}))
    else:
        p = load_params(a.params)
        md = S.rim_training_model(a.n, a.seed)
        vel, rho = md["vel"], md["rho"]
        dt = S.cfl_dt(10.0, 4500.0)
        c = a.n // 2
        r = reflection(vel, rho, (c, c, 8), a.nt, dt, p)
        r["choice"] = choose_boundary(r)
        print(json.dumps(r))


if __name__ == "__main__":
    _main()
