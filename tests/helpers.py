"""Seeded synthetic models and comparison helpers shared by the tests."""
import numpy as np

NPML_REF = {"2o": 50, "iso": 20, "vti": 20, "tti": 40}
MODELS = {"2o": ("vel",), "iso": ("vel", "rho"), "vti": ("vel", "rho", "eps", "del"),
          "tti": ("vel", "eps", "del", "theta", "phi")}


def smooth_field(rng, shape, lo, hi, sigma=2.0):
    from scipy.ndimage import gaussian_filter
    a = gaussian_filter(rng.standard_normal(shape), sigma=sigma, mode="reflect")
    a = (a - a.min()) / max(a.max() - a.min(), 1e-12)
    return (lo + (hi - lo) * a).astype(np.float32)


def make_models(engine, nx, ny, nz, seed, vlo=1800.0, vhi=3000.0):
    """Smooth seeded models, shape (ny, nx, nz) — z fastest on disk."""
    rng = np.random.default_rng(seed)
    shape = (ny, nx, nz)
    vel = smooth_field(rng, shape, vlo, vhi)
    m = {"vel": vel, "rho": (310.0 * vel.astype(np.float64) ** 0.25).astype(np.float32)}
    eps = smooth_field(rng, shape, 0.05, 0.25)
    m["eps"] = eps
    m["del"] = np.minimum(smooth_field(rng, shape, 0.0, 0.12), eps).astype(np.float32)
    m["theta"] = smooth_field(rng, shape, 0.0, 0.4, sigma=4.0)
    m["phi"] = smooth_field(rng, shape, 0.2, 0.8, sigma=4.0)
    return {k: m[k] for k in MODELS[engine]}


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (d if d > 0 else 1.0))


def decimate(rec, jx, jy, jt):
    """The reference's record-file order: iy (step jy), ix (step jx), it (step jt)."""
    return np.ascontiguousarray(rec[::jy, ::jx, ::jt]).ravel()
