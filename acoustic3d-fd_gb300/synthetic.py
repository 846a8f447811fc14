"""Seeded synthetic models of the five benchmark configurations.

The reference ships no models: readmodel.py's Model only writes constant fields
(readmodel.py:20-73).  These generators give the seeded fields the benchmarks and
tests use, as host arrays in the reference's file order (z fastest, then x, then
y; numpy shape (ny, nx, nz)), ready for Model.write_* or the a3d_* API.

* smooth fields: standard-normal noise (numpy default_rng(seed)), Gaussian
  smoothing (sigma 8 cells, reflecting edges), mapped linearly onto [lo, hi];
* density by Gardner's relation rho = 310 v^0.25;
* delta = min(delta', epsilon) so that delta <= epsilon.
"""
from __future__ import annotations

import numpy as np


def smooth_field3(nx, ny, nz, seed, lo, hi, sigma=8.0):
    """Gaussian-smoothed seeded noise mapped linearly to [lo, hi], shape (ny, nx, nz)."""
    from scipy.ndimage import gaussian_filter
    rng = np.random.default_rng(seed)
    a = gaussian_filter(rng.standard_normal((ny, nx, nz)).astype(np.float32), sigma=sigma, mode="reflect")
    a = (a - a.min()) / (a.max() - a.min())
    return (lo + (hi - lo) * a).astype(np.float32)


def gardner(vel):
    """rho = 310 v^0.25 (kg/m^3, v in m/s)."""
    return (310.0 * np.asarray(vel).astype(np.float64) ** 0.25).astype(np.float32)


def cfl_dt(d, vmax, factor=1.0):
    """dt = 0.4 d / (vmax factor) as float32 (factor sqrt(1.6) for VTI and TTI)."""
    return float(np.float32(0.4 * d / (vmax * factor)))


def layered_2o(n=128):
    """2nd-order three-layer model: 1500 m/s above z = 40, 2500 to z = 85, 3500 below."""
    z = np.arange(n)
    col = np.where(z < 40, 1500.0, np.where(z < 85, 2500.0, 3500.0)).astype(np.float32)
    return {"vel": np.broadcast_to(col, (n, n, n)).copy()}


def iso_model(n=256, seed=2, vmax=4500.0):
    """Isotropic model with density: smooth velocity 1500..vmax (seed 2), Gardner density."""
    vel = smooth_field3(n, n, n, seed, 1500.0, vmax)
    return {"vel": vel, "rho": gardner(vel)}


def vti_model(nx=384, ny=384, nz=256, vmax=4500.0):
    """VTI model: v 1500..vmax (seed 3), Gardner density, epsilon 0..0.3 (seed 4),
    delta = min(delta', epsilon) with delta' 0..0.15 (seed 5)."""
    vel = smooth_field3(nx, ny, nz, 3, 1500.0, vmax)
    eps = smooth_field3(nx, ny, nz, 4, 0.0, 0.3)
    dl = np.minimum(smooth_field3(nx, ny, nz, 5, 0.0, 0.15), eps).astype(np.float32)
    return {"vel": vel, "rho": gardner(vel), "eps": eps, "del": dl}


def vti_shot_grid(k=8, first=24, step=48, z=2):
    """Shots on a k x k surface grid: x, y in first + step * i."""
    return [(first + step * i, first + step * j, z) for j in range(k) for i in range(k)]


def tti_model(nx=512, ny=512, nz=320, vmax=5000.0):
    """TTI model: v 1500..vmax (seed 7), epsilon 0..0.3 (seed 8), delta <= epsilon in
    0..0.15 (seed 9), tilt 0..45 deg (seed 10) and azimuth 0..360 deg (seed 11), in
    radians (the reference takes cos() of the file values directly)."""
    vel = smooth_field3(nx, ny, nz, 7, 1500.0, vmax)
    eps = smooth_field3(nx, ny, nz, 8, 0.0, 0.3)
    dl = np.minimum(smooth_field3(nx, ny, nz, 9, 0.0, 0.15), eps).astype(np.float32)
    th = smooth_field3(nx, ny, nz, 10, 0.0, np.pi / 4)
    ph = smooth_field3(nx, ny, nz, 11, 0.0, 2 * np.pi)
    return {"vel": vel, "eps": eps, "del": dl, "theta": th, "phi": ph}


def tti_windows(nx=512, ny=512, nz=320, count=48, lo=160, hi=320, seed=12, depth=2):
    """count apertures with sizes uniform per axis in [lo, hi] and origins uniform
    inside the model (seed 12), each with its shot at the window centre, z = depth.
    Returns (windows [(x0, y0, z0, wx, wy, wz)], shots [(sx, sy, sz)])."""
    rng = np.random.default_rng(seed)
    wins, shots = [], []
    for _ in range(count):
        wx, wy, wz = (int(v) for v in rng.integers(lo, hi + 1, size=3))
        x0 = int(rng.integers(0, nx - wx + 1))
        y0 = int(rng.integers(0, ny - wy + 1))
        z0 = int(rng.integers(0, nz - wz + 1))
        wins.append((x0, y0, z0, wx, wy, wz))
        shots.append((x0 + wx // 2, y0 + wy // 2, z0 + depth))
    return wins, shots


def rim_training_model(n, seed, vmax=4500.0, sigma=8.0):
    """One training model of the learned rim (seeds 1000..1199): smooth velocity
    1500..vmax, Gardner density."""
    vel = smooth_field3(n, n, n, seed, 1500.0, vmax, sigma)
    return {"vel": vel, "rho": gardner(vel)}
