"""ctypes binding of the CPU oracle (oracle/a3d_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` as the oracle.  The product never imports it.

The oracle restates the reference engines (paths relative to the reference
project): src/Toa_3dfd_cuda.cu (2nd order), src/Toa_gpu_3diso_fd_1orderfunciton.cu
(isotropic), src/Toa_gpu_3dvti_fd_1orderfunciton.cu (VTI) and
src/Toa_gpu_3dtti_fd_1orderfunciton.cu (TTI).  Records come back as numpy arrays of
shape (ny, nx, nt) — the reference's internal record layout, it fastest.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liba3d_oracle.so")

# reference absorber widths and receiver depths
NPD_2ORDER = 50      # Toa_3dfd_cuda.cu:19
NPML_ISO = 20        # ..iso..:395
NPML_VTI = 20        # ..vti..:414
NPML_TTI = 40        # ..tti..:418


class OracleCfg(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("dx", ctypes.c_float), ("dy", ctypes.c_float), ("dz", ctypes.c_float),
        ("sx", ctypes.c_int), ("sy", ctypes.c_int), ("sz", ctypes.c_int),
        ("nt", ctypes.c_int),
        ("dt", ctypes.c_float), ("fm", ctypes.c_float),
        ("wtype", ctypes.c_int), ("npml", ctypes.c_int), ("rec_z", ctypes.c_int),
        ("mute", ctypes.c_int), ("snap_every", ctypes.c_int), ("snap_skip0", ctypes.c_int),
        ("form", ctypes.c_int), ("threads", ctypes.c_int),
        ("store", ctypes.c_int), ("sig_v_log2", ctypes.c_int), ("sig_p_log2", ctypes.c_int),
    ]


@dataclass
class Shot:
    """One shot's geometry and run settings (model arrays are passed separately)."""
    nx: int
    ny: int
    nz: int
    dx: float = 10.0
    dy: float = 10.0
    dz: float = 10.0
    sx: int = 0
    sy: int = 0
    sz: int = 0
    nt: int = 100
    dt: float = 1e-3
    fm: float = 20.0
    wtype: int = 1
    npml: int = 20
    rec_z: int = 1
    mute: bool = False
    snap_every: int = 0
    snap_skip0: bool = False
    form: int = 0
    threads: int = 0
    store: int = 0          # storage emulated (float oracle, engine form): 1 bf16, 2 fp16, 4 FP16V; 5 / 6 24-bit
                            # floats (every field / u, v, w only), a format no engine stores yet
    sig_v_log2: int = 0     # float16 scales, log2 (the engine reports them)
    sig_p_log2: int = 0
    extra: dict = field(default_factory=dict)

    def cfg(self) -> OracleCfg:
        return OracleCfg(self.nx, self.ny, self.nz, self.dx, self.dy, self.dz,
                         self.sx, self.sy, self.sz, self.nt, self.dt, self.fm,
                         self.wtype, self.npml, self.rec_z, int(self.mute),
                         self.snap_every, int(self.snap_skip0), self.form, self.threads, self.store,
                         self.sig_v_log2, self.sig_p_log2)

    def n_snaps(self) -> int:
        if self.snap_every <= 0:
            return 0
        return sum(1 for it in range(self.nt)
                   if it % self.snap_every == 0 and not (self.snap_skip0 and it == 0))


_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle library with make (gcc, OpenMP)."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        fp = ctypes.POINTER(ctypes.c_float)
        dp = ctypes.POINTER(ctypes.c_double)
        cp = ctypes.POINTER(OracleCfg)
        for name, nin in (("2o", 1), ("iso", 2), ("vti", 4), ("tti", 5)):
            for suf, op in (("f32", fp), ("f64", dp)):
                fn = getattr(L, f"a3d_oracle_{name}_{suf}")
                fn.argtypes = [cp] + [fp] * nin + [op, op]
                fn.restype = ctypes.c_int
        L.a3d_oracle_ricker2o.argtypes = [ctypes.c_int, ctypes.c_float, ctypes.c_float]
        L.a3d_oracle_ricker2o.restype = ctypes.c_float
        L.a3d_oracle_wavelet.argtypes = [ctypes.c_int, ctypes.c_float, ctypes.c_float]
        L.a3d_oracle_wavelet.restype = ctypes.c_float
        L.a3d_oracle_round_f16.argtypes = [ctypes.c_float]
        L.a3d_oracle_round_f16.restype = ctypes.c_float
        L.a3d_oracle_round_bf16.argtypes = [ctypes.c_float]
        L.a3d_oracle_round_bf16.restype = ctypes.c_float
        L.a3d_oracle_round_f24.argtypes = [ctypes.c_float]
        L.a3d_oracle_round_f24.restype = ctypes.c_float
        L.a3d_oracle_d0.argtypes = [fp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_float, ctypes.c_float, ctypes.c_float]
        L.a3d_oracle_d0.restype = ctypes.c_float
        L.a3d_oracle_pml.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_int, ctypes.c_int,
                                     fp, fp, fp, fp]
        L.a3d_oracle_pml.restype = None
        L.a3d_oracle_mute_nt.argtypes = [ctypes.c_int] * 5 + [ctypes.c_float] * 6
        L.a3d_oracle_mute_nt.restype = ctypes.c_int
        _lib = L
    return _lib


def _fptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _model(a, s: Shot):
    a = np.ascontiguousarray(a, dtype=np.float32)
    assert a.size == s.nx * s.ny * s.nz, "model size mismatch"
    return a


def run(engine: str, s: Shot, models: dict, precision: str = "f32", snaps: bool = False):
    """Run one shot on the oracle.

    engine: "2o" | "iso" | "vti" | "tti"; models: dict with the arrays the engine
    reads ("vel", "rho", "eps", "del", "theta", "phi"), each flat or (ny, nx, nz).
    Returns (record[ny, nx, nt], snapshots[nsnap, ny, nx, nz] or None).
    """
    names = {"2o": ("vel",), "iso": ("vel", "rho"), "vti": ("vel", "rho", "eps", "del"),
             "tti": ("vel", "eps", "del", "theta", "phi")}[engine]
    arrs = [_model(models[n], s) for n in names]
    dt = np.float32 if precision == "f32" else np.float64
    rec = np.zeros((s.ny, s.nx, s.nt), dtype=dt)
    ns = s.n_snaps() if snaps else 0
    snap = np.zeros((max(ns, 1), s.ny, s.nx, s.nz), dtype=dt) if ns else None
    optr = ctypes.POINTER(ctypes.c_float if precision == "f32" else ctypes.c_double)
    fn = getattr(lib(), f"a3d_oracle_{engine}_{precision}")
    c = s.cfg()
    rc = fn(ctypes.byref(c), *[_fptr(a) for a in arrs],
            rec.ctypes.data_as(optr),
            snap.ctypes.data_as(optr) if snap is not None else ctypes.cast(None, optr))
    if rc != 0:
        raise RuntimeError(f"oracle {engine} failed with status {rc}")
    return rec, snap


def pml_profile(dt, d0, n, npml):
    L = lib()
    nn = n + 2 * npml
    out = [np.zeros(nn, np.float32) for _ in range(4)]
    L.a3d_oracle_pml(dt, d0, n, npml, *[_fptr(a) for a in out])
    return out


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0))
