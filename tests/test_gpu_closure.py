"""Learned absorbing rim: teacher taps, the student step, the closure kernels and
their gradients against a PyTorch float32 restatement (tests/closure_ref.py), the
training loop, and the learned-rim engine."""
import os

import numpy as np
import pytest

import closure_ref as R

pytestmark = pytest.mark.gpu

NX, NY, NZ = 14, 12, 16
DX, FM, VMAX = 10.0, 20.0, 4500.0
WIDE = 30


def _model(seed):
    import learned_abc as L
    vel = L.smooth_velocity(NX, NY, NZ, seed, 1500.0, VMAX, sigma=3.0)
    return vel, L.gardner(vel)


def _closure_with_samples(engine_lib, seeds=(5,), taps=(62, 63)):
    """Closure object with consecutive teacher pairs (t, t+1) for t in taps."""
    import a3d
    dt = float(np.float32(0.4 * DX / VMAX))
    cl = a3d.Closure(NX, NY, NZ)
    steps = sorted(set(s for t in taps for s in (t, t + 1)))
    fb = cl.state_floats() * 4
    for seed in seeds:
        vel, rho = _model(seed)
        cfg = a3d.make_config("iso", NX, NY, NZ, DX, DX, DX, nt=max(steps) + 1, dt=dt, fm=FM, npml=WIDE, tile_x=8)
        e = a3d.Engine(cfg, {"vel": vel, "rho": rho})
        buf = cl.staging(len(steps))
        e.set_tap(steps, WIDE - a3d.CLOSURE_PAD, buf)
        e.run_device(NX // 2, NY // 2, NZ // 2)
        e.close()
        mid = cl.add_model(vel, rho, DX, DX, DX, dt)
        for t in taps:
            cl.add_sample(mid, buf + steps.index(t) * fb, buf + steps.index(t + 1) * fb)
    return cl, dt


def _scales(seed, dt):
    vel, rho = _model(seed)
    vp, rp = R.pad_model(vel), R.pad_model(rho)
    zinv, kap = R.scales(vp, rp, np.float32(dt) / np.float32(DX))
    return vp, rp, zinv, kap


def _rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-30))


def test_taps_match_snapshots(engine_lib):
    """A tap of P equals the engine's own snapshot of P over the model window."""
    import a3d
    vel, rho = _model(5)
    dt = float(np.float32(0.4 * DX / VMAX))
    cfg = a3d.make_config("iso", NX, NY, NZ, DX, DX, DX, nt=61, dt=dt, fm=FM, npml=WIDE, tile_x=8)
    cl = a3d.Closure(NX, NY, NZ)
    buf = cl.staging(1)
    e = a3d.Engine(cfg, {"vel": vel, "rho": rho})
    e.set_tap([60], WIDE - a3d.CLOSURE_PAD, buf)
    rec, snaps = e.run(NX // 2, NY // 2, NZ // 2, snap_every=60, snap_skip0=True)
    e.close()
    mid = cl.add_model(vel, rho, DX, DX, DX, dt)
    cl.add_sample(mid, buf, buf)
    _, t = cl.teacher(0)
    p = a3d.CLOSURE_PAD
    assert np.array_equal(t[3][p:-p, p:-p, p:-p], snaps[0])
    assert np.any(t[0] != 0) and np.any(t[3][:p] != 0)  # the rim cells carry the wave
    cl.close()


def test_student_step_is_the_undamped_update(engine_lib):
    cl, dt = _closure_with_samples(engine_lib, taps=(62, 63))
    _, T0 = cl.teacher(0)
    X1, _ = cl.teacher(1)                 # step(S_63), S_63 = sample 0's target
    vp, rp, _, _ = _scales(5, dt)
    ref = R.std_step(T0, rp, vp, dt / DX, dt / DX, dt / DX)
    for k in range(4):
        scale = np.abs(ref[k]).max()
        assert scale > 0
        assert np.abs(X1[k] - ref[k]).max() <= 2e-5 * scale, k
    assert not np.any(X1[:, :4]) and not np.any(X1[:, :, :, -4:])  # never-updated cells stay zero
    cl.close()


def _params(seed=3, w2_scale=30.0):
    import learned_abc as L
    p = L.init_params(seed)
    p[L.NW1:L.NW1 + L.NW2] *= w2_scale
    rng = np.random.default_rng(seed + 1)
    p[L.NW1 + L.NW2:] = rng.uniform(0.5, 1.5, L.NG)
    return p


def test_closure_forward_matches_torch(engine_lib):
    cl, dt = _closure_with_samples(engine_lib)
    p = _params()
    cl.set_params(p)
    d, _, _ = cl.eval(0)
    X, _ = cl.teacher(0)
    _, _, zinv, kap = _scales(5, dt)
    ref = R.closure(X, zinv, kap, p)
    mask = R.rim_mask(X.shape[1:])
    assert not np.any(d[:, ~mask])
    for k in range(4):
        assert np.abs(ref[k][mask]).max() > 0
        assert _rel(d[k][mask], ref[k][mask]) < 2e-3, k
    cl.close()


def test_tensor_core_closure_matches(engine_lib):
    """The tcgen05 kernels give the CUDA-core kernels' correction (float summation
    order apart) on every rim cell of every face, edges and corners included."""
    cl, dt = _closure_with_samples(engine_lib)
    p = _params()
    cl.set_params(p)
    d, _, _ = cl.eval(0)
    dt_ = cl.eval_tc(0)
    X, _ = cl.teacher(0)
    _, _, zinv, kap = _scales(5, dt)
    ref = R.closure(X, zinv, kap, p)
    mask = R.rim_mask(X.shape[1:])
    assert not np.any(dt_[:, ~mask])
    for k in range(4):
        assert _rel(dt_[k][mask], d[k][mask]) < 2e-3, k
        assert _rel(dt_[k][mask], ref[k][mask]) < 2e-3, k
    cl.close()


def test_closure_gradient_matches_torch(engine_lib):
    cl, dt = _closure_with_samples(engine_lib)
    p = _params()
    cl.set_params(p)
    _, g, loss = cl.eval(0)
    X, T = cl.teacher(0)
    _, _, zinv, kap = _scales(5, dt)
    lref, gref = R.loss_and_grad(X, T, zinv, kap, p)
    assert abs(loss - lref) <= 1e-3 * lref
    import learned_abc as L
    for name, sl in (("W1", slice(0, L.NW1)), ("W2", slice(L.NW1, L.NW1 + L.NW2)), ("G", slice(L.NW1 + L.NW2, None))):
        assert _rel(g[sl], gref[sl]) < 2e-2, name
    cl.close()


def test_training_lowers_the_loss(engine_lib):
    import learned_abc as L
    cl, _ = _closure_with_samples(engine_lib, seeds=(5, 6, 7), taps=(62, 80, 100))
    cl.set_params(L.init_params(0))
    losses = cl.train(20, 3, 2e-3, seed=1)
    assert np.all(np.isfinite(losses))
    assert losses[-1] < 0.9 * losses[0], losses
    assert np.all(np.isfinite(cl.params()))
    cl.close()


def test_learned_rim_engine(engine_lib):
    """The learned-rim engine needs a closure, runs with one (zero weights leave the
    rim undamped), and is built for the isotropic FP32 engine only."""
    import a3d
    import learned_abc as L
    vel, rho = _model(5)
    dt = float(np.float32(0.4 * DX / VMAX))
    shot = (NX // 2, NY // 2, NZ // 2)
    cfg = a3d.make_config("iso", NX, NY, NZ, DX, DX, DX, nt=150, dt=dt, fm=FM, boundary="learned")
    e = a3d.Engine(cfg, {"vel": vel, "rho": rho})
    with pytest.raises(a3d.A3DError):
        e.run(*shot)                          # no closure installed
    e.set_closure(np.zeros(a3d.CLOSURE_NPARAM, np.float32))
    r0 = e.run(*shot)
    e.set_closure(L.init_params(0))
    e.set_profiling(True)
    r1 = e.run(*shot)
    ms, n = e.closure_times()
    e.close()
    assert n == 150 and ms > 0
    # the CUDA-core closure gives the same record to float summation order
    os.environ["A3D_CLOSURE_SIMT"] = "1"
    try:
        e = a3d.Engine(cfg, {"vel": vel, "rho": rho})
        e.set_closure(L.init_params(0))
        r2 = e.run(*shot)
        e.close()
    finally:
        os.environ.pop("A3D_CLOSURE_SIMT", None)
    assert _rel(r2, r1) < 1e-3
    assert np.all(np.isfinite(r0)) and np.all(np.isfinite(r1))
    assert not np.array_equal(r0, r1)
    with pytest.raises(a3d.A3DError):         # the learned rim is isotropic FP32 only
        a3d.Engine(a3d.make_config("vti", NX, NY, NZ, nt=10, boundary="learned"),
                   {"vel": vel, "rho": rho, "eps": vel * 0, "del": vel * 0})
