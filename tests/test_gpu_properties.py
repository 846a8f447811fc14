"""Physical and cross-engine properties of the records, on the GPU path.

Each test checks a fact that holds whatever the grid size, so the isotropic one
runs at the 256^3, 2000-step size of the isotropic benchmark:

* TTI with zero tilt and azimuth is VTI with unit density: cos 0 = 1 and sin 0 = 0
  reduce the rotated derivatives of ..tti..:101-103 and 184-186 to the axis
  derivatives of ..vti..:113-119 and 183-199, and 1 / rho = 1 removes the density,
  so with the same PML width the two engines give the same record, bit for bit.
* An isotropic shot in a model that depends on depth only, with the source on the
  x = y diagonal and dx = dy, is symmetric under the swap of x and y.  The two
  orders of the pressure update's x and y terms round differently, so the record
  and its transpose agree to float rounding (rel-L2 below 1e-5; measured 1.1e-6),
  not bit for bit.
* In a homogeneous medium the delay between the traces of two receivers is their
  difference in distance from the source over the velocity (within 1 ms; measured
  0.15 ms off on a 49 ms delay).
* The PML takes the energy out: once the wave has left the model, the pressure
  energy inside it is a tiny fraction of its peak.

It also checks that the geometry checks made after the device is chosen report the
offending value.
"""
import numpy as np
import pytest

from helpers import make_models, rel_l2

pytestmark = pytest.mark.gpu


def test_tti_zero_tilt_equals_vti_unit_density(engine_lib):
    import a3d
    nx, ny, nz, nt = 40, 36, 44, 200
    m = make_models("vti", nx, ny, nz, seed=41)
    vti = dict(m, rho=np.ones_like(m["vel"]))
    zero = np.zeros_like(m["vel"])
    tti = {"vel": m["vel"], "eps": m["eps"], "del": m["del"], "theta": zero, "phi": zero}
    recs = []
    for phys, models in (("vti", vti), ("tti", tti)):
        cfg = a3d.make_config(phys, nx, ny, nz, nt=nt, dt=1e-3, fm=25.0, npml=20)
        e = a3d.Engine(cfg, models)
        try:
            recs.append(e.run(19, 17, 5))
        finally:
            e.close()
    assert np.abs(recs[0]).max() > 0
    assert np.array_equal(recs[0], recs[1])


def test_iso_shot_is_symmetric_under_x_y_swap_full_size(engine_lib):
    import a3d
    n, nt, dx = 256, 2000, 10.0
    z = np.arange(n, dtype=np.float64)
    v1 = 1500.0 + 3000.0 * (0.5 + 0.5 * np.tanh((z - 120.0) / 30.0))  # depth profile, 1500-4500 m/s
    vel = np.broadcast_to(v1.astype(np.float32), (n, n, n)).copy()
    rho = (310.0 * vel.astype(np.float64) ** 0.25).astype(np.float32)
    dt = float(np.float32(0.4 * dx / 4500.0))
    cfg = a3d.make_config("iso", n, n, n, dx=dx, dy=dx, dz=dx, nt=nt, dt=dt, fm=20.0, npml=20)
    e = a3d.Engine(cfg, {"vel": vel, "rho": rho})
    try:
        rec = e.run(n // 2, n // 2, 8)  # [y][x][t]
    finally:
        e.close()
    assert np.isfinite(rec).all() and np.abs(rec).max() > 0
    err = rel_l2(rec, rec.transpose(1, 0, 2))
    assert err < 1e-5, err


def _lag_seconds(a, b, dt):
    """Delay of trace b behind trace a from the peak of their cross-correlation,
    refined by a parabola through the peak and its neighbours."""
    c = np.correlate(b.astype(np.float64), a.astype(np.float64), mode="full")
    k = int(np.argmax(c))
    frac = 0.0
    if 0 < k < len(c) - 1:
        y0, y1, y2 = c[k - 1], c[k], c[k + 1]
        den = y0 - 2 * y1 + y2
        frac = 0.5 * (y0 - y2) / den if den != 0 else 0.0
    return (k - (len(a) - 1) + frac) * dt


def test_homogeneous_moveout_is_distance_over_velocity(engine_lib):
    import a3d
    nx, ny, nz, nt, d, vp, dt = 96, 96, 64, 600, 10.0, 2000.0, 1e-3
    models = {"vel": np.full((ny, nx, nz), vp, np.float32), "rho": np.full((ny, nx, nz), 1000.0, np.float32)}
    cfg = a3d.make_config("iso", nx, ny, nz, dx=d, dy=d, dz=d, nt=nt, dt=dt, fm=20.0, npml=20)
    sx, sy, sz = 48, 48, 41  # source cells (47, 47, 40) and (47, 47, 42): the dipole's centre is cell 41
    e = a3d.Engine(cfg, models)
    try:
        rec = e.run(sx, sy, sz)
    finally:
        e.close()
    ix0, iy0, off = sx - 1, sy - 1, 30
    h = 41 * d  # depth of the dipole's centre below the receivers (model z = 0)
    r1, r2 = h, np.hypot(h, off * d)
    lag = _lag_seconds(rec[iy0, ix0], rec[iy0, ix0 + off], dt)
    assert abs(lag - (r2 - r1) / vp) < 1e-3, (lag, (r2 - r1) / vp)
    # the same along y
    lag_y = _lag_seconds(rec[iy0, ix0], rec[iy0 + off, ix0], dt)
    assert abs(lag_y - (r2 - r1) / vp) < 1e-3, (lag_y, (r2 - r1) / vp)


def test_pml_takes_the_energy_out(engine_lib):
    import a3d
    n, nt, d, vp, dt, every = 64, 1200, 10.0, 2000.0, 1e-3, 50
    models = {"vel": np.full((n, n, n), vp, np.float32), "rho": np.full((n, n, n), 1000.0, np.float32)}
    cfg = a3d.make_config("iso", n, n, n, dx=d, dy=d, dz=d, nt=nt, dt=dt, fm=20.0, npml=20)
    e = a3d.Engine(cfg, models)
    try:
        _, snaps = e.run(n // 2, n // 2, n // 2, snap_every=every)
    finally:
        e.close()
    energy = (snaps.astype(np.float64) ** 2).reshape(len(snaps), -1).sum(axis=1)
    peak = energy.max()
    assert peak > 0
    # the wave crosses the 640 m model in 0.32 s; by 1.15 s it has left it (measured
    # on a GB300: 3e-10 of the peak)
    assert energy[-1] < 1e-6 * peak, energy[-1] / peak


@pytest.mark.parametrize("physics,kw,msg", [("2o", {"rec_z": 12}, "receiver depth 12 outside the model"),
                                            ("iso", {"npml": 4}, "PML width 4 below 6 cells")])
def test_engine_create_rejects_bad_geometry(engine_lib, physics, kw, msg):
    """Geometry checks that run after the device is chosen return A3D_E_ARG with the
    offending value in the message (the engine is released before the message is
    formatted)."""
    import ctypes
    import a3d
    cfg = a3d.make_config(physics, 12, 12, 12, nt=10, **kw)
    h = ctypes.c_void_p()
    m = {k: np.full((12, 12, 12), 2000.0, np.float32) for k in ("vel", "rho")}
    rc = a3d.lib().a3d_engine_create(ctypes.byref(h), ctypes.byref(cfg), a3d._fptr(m["vel"]), a3d._fptr(m["rho"]),
                                     *[a3d._fptr(None)] * 4, 0)
    assert rc == a3d.A3D_E_ARG
    assert msg in a3d.last_error()
