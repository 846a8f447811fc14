"""ctypes binding of the engine library (lib/libacoustic3d.so, include/acoustic3d.h).

There is no fallback: if the library is missing or cannot be loaded, every entry
point raises.  Build it with ``python acoustic3d-fd_gb300/build.py``.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(HERE, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libacoustic3d.so")
LEGACY_LIBS = {"2order": "acoustic2order.so", "1order": "acoustic1order.so",
               "vti": "acoustic1vti.so", "tti": "acoustic1tti.so"}

ORDER2, ISO, VTI, TTI = 0, 1, 2, 3
FP32, BF16, FP16, FP64, FP16V = 0, 1, 2, 3, 4  # FP16V: VTI / TTI, float16 u, v, w with float P, Q
PHYSICS = {"2o": ORDER2, "iso": ISO, "vti": VTI, "tti": TTI}
MODEL_NAMES = ("vel", "rho", "eps", "del", "theta", "phi")
READS = {ORDER2: ("vel",), ISO: ("vel", "rho"), VTI: ("vel", "rho", "eps", "del"),
         TTI: ("vel", "eps", "del", "theta", "phi")}

A3D_OK, A3D_E_ARG, A3D_E_IO, A3D_E_CUDA, A3D_E_NOMEM, A3D_E_KERNEL, A3D_E_UNSUPPORTED = range(7)


class Config(ctypes.Structure):
    _fields_ = [("physics", ctypes.c_int),
                ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("dx", ctypes.c_float), ("dy", ctypes.c_float), ("dz", ctypes.c_float),
                ("nt", ctypes.c_int), ("dt", ctypes.c_float), ("fm", ctypes.c_float),
                ("wtype", ctypes.c_int), ("npml", ctypes.c_int), ("rec_z", ctypes.c_int),
                ("mute", ctypes.c_int), ("storage", ctypes.c_int), ("tile_x", ctypes.c_int),
                ("boundary", ctypes.c_int), ("batch", ctypes.c_int)]


BOUNDARY_PML, BOUNDARY_LEARNED = 0, 1
BOUNDARIES = {"pml": BOUNDARY_PML, "learned": BOUNDARY_LEARNED}
CLOSURE_NPARAM = 27792   # W1 [32][8][27], W2 [6][4][32][27], G [6][6][4]
CLOSURE_PAD = 10         # rim-grid padding per face: 6 rim cells + 4 never updated


class ShotPos(ctypes.Structure):
    _fields_ = [("sx", ctypes.c_int), ("sy", ctypes.c_int), ("sz", ctypes.c_int)]


class Window(ctypes.Structure):
    _fields_ = [("x0", ctypes.c_int), ("y0", ctypes.c_int), ("z0", ctypes.c_int),
                ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int)]


class Problem(ctypes.Structure):
    _fields_ = [("cfg", Config)] + [(n, ctypes.POINTER(ctypes.c_float)) for n in
                                     ("vel", "rho", "eps", "del_", "theta", "phi")]


class Opts(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("windows", ctypes.POINTER(Window)), ("graph", ctypes.c_int),
                ("recs_host", ctypes.POINTER(ctypes.c_float)), ("rec_offsets", ctypes.POINTER(ctypes.c_size_t)),
                ("ms", ctypes.POINTER(ctypes.c_double))]


class A3DError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"acoustic3d status {code}: {msg}")
        self.code = code


_lib = None
_FP = ctypes.POINTER(ctypes.c_float)


def lib() -> ctypes.CDLL:
    """Load the engine library (raises if it is missing)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run acoustic3d-fd_gb300/build.py")
        L = ctypes.CDLL(LIB_PATH)
        vp = ctypes.c_void_p
        L.a3d_engine_create.argtypes = [ctypes.POINTER(vp), ctypes.POINTER(Config)] + [_FP] * 6 + [ctypes.c_int]
        L.a3d_engine_create.restype = ctypes.c_int
        L.a3d_engine_destroy.argtypes = [vp]
        L.a3d_engine_destroy.restype = ctypes.c_int
        L.a3d_engine_run.argtypes = [vp, ctypes.POINTER(ShotPos), _FP, ctypes.c_int, ctypes.c_int, _FP,
                                     ctypes.POINTER(ctypes.c_double)]
        L.a3d_engine_run.restype = ctypes.c_int
        L.a3d_engine_run_device.argtypes = [vp, ctypes.POINTER(ShotPos), vp, ctypes.POINTER(ctypes.c_double)]
        L.a3d_engine_run_device.restype = ctypes.c_int
        L.a3d_engine_run_shots.argtypes = [vp, ctypes.POINTER(ShotPos), ctypes.c_int, _FP,
                                           ctypes.POINTER(ctypes.c_double)]
        L.a3d_engine_run_shots.restype = ctypes.c_int
        L.a3d_engine_copy_record.argtypes = [vp, ctypes.c_int, _FP]
        L.a3d_engine_copy_record.restype = ctypes.c_int
        L.a3d_engine_record_device.argtypes = [vp]
        L.a3d_engine_record_device.restype = vp
        L.a3d_engine_device_bytes.argtypes = [vp]
        L.a3d_engine_device_bytes.restype = ctypes.c_size_t
        L.a3d_forward_host.argtypes = [ctypes.POINTER(Config)] + [_FP] * 6 + [ctypes.POINTER(ShotPos),
                                                                               ctypes.c_int, _FP, ctypes.c_int]
        L.a3d_forward_host.restype = ctypes.c_int
        L.a3d_engine_set_profiling.argtypes = [vp, ctypes.c_int]
        L.a3d_engine_set_profiling.restype = ctypes.c_int
        L.a3d_engine_kernel_times.argtypes = [vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong)]
        L.a3d_engine_kernel_times.restype = ctypes.c_int
        L.a3d_engine_describe.argtypes = [vp, ctypes.c_char_p, ctypes.c_size_t]
        L.a3d_engine_describe.restype = ctypes.c_int
        L.a3d_run_batch.argtypes = [ctypes.POINTER(Problem), ctypes.POINTER(ShotPos), ctypes.c_int,
                                    ctypes.POINTER(Opts)]
        L.a3d_run_batch.restype = ctypes.c_int
        L.a3d_engine_set_closure.argtypes = [vp, _FP, ctypes.c_size_t]
        L.a3d_engine_set_closure.restype = ctypes.c_int
        L.a3d_engine_set_tap.argtypes = [vp, ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_int, vp]
        L.a3d_engine_set_tap.restype = ctypes.c_int
        L.a3d_engine_closure_times.argtypes = [vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong)]
        L.a3d_engine_closure_times.restype = ctypes.c_int
        L.a3d_closure_create.argtypes = [ctypes.POINTER(vp), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.a3d_closure_create.restype = ctypes.c_int
        L.a3d_closure_destroy.argtypes = [vp]
        L.a3d_closure_destroy.restype = ctypes.c_int
        L.a3d_closure_set_params.argtypes = [vp, _FP, ctypes.c_size_t]
        L.a3d_closure_set_params.restype = ctypes.c_int
        L.a3d_closure_get_params.argtypes = [vp, _FP, ctypes.c_size_t]
        L.a3d_closure_get_params.restype = ctypes.c_int
        L.a3d_closure_add_model.argtypes = [vp, _FP, _FP] + [ctypes.c_float] * 4 + [ctypes.POINTER(ctypes.c_int)]
        L.a3d_closure_add_model.restype = ctypes.c_int
        L.a3d_closure_add_sample.argtypes = [vp, ctypes.c_int, vp, vp]
        L.a3d_closure_add_sample.restype = ctypes.c_int
        L.a3d_closure_num_samples.argtypes = [vp]
        L.a3d_closure_num_samples.restype = ctypes.c_int
        L.a3d_closure_set_decay.argtypes = [vp, ctypes.c_float]
        L.a3d_closure_set_decay.restype = ctypes.c_int
        L.a3d_closure_staging.argtypes = [vp, ctypes.c_int]
        L.a3d_closure_staging.restype = vp
        L.a3d_closure_train.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_ulonglong, _FP]
        L.a3d_closure_train.restype = ctypes.c_int
        L.a3d_closure_eval.argtypes = [vp, ctypes.c_int, _FP, _FP, _FP]
        L.a3d_closure_eval.restype = ctypes.c_int
        L.a3d_closure_eval_tc.argtypes = [vp, ctypes.c_int, _FP]
        L.a3d_closure_eval_tc.restype = ctypes.c_int
        L.a3d_closure_teacher.argtypes = [vp, ctypes.c_int, _FP, _FP]
        L.a3d_closure_teacher.restype = ctypes.c_int
        L.a3d_last_error.argtypes = []
        L.a3d_last_error.restype = ctypes.c_char_p
        _lib = L
    return _lib


def last_error() -> str:
    return lib().a3d_last_error().decode(errors="replace")


def _check(rc):
    if rc != A3D_OK:
        raise A3DError(rc, last_error())


def _fptr(a):
    if a is None:
        return ctypes.cast(None, _FP)
    return a.ctypes.data_as(_FP)


def make_config(physics, nx, ny, nz, dx=10.0, dy=10.0, dz=10.0, nt=100, dt=1e-3, fm=20.0, wtype=1,
                npml=0, rec_z=-1, mute=False, storage=FP32, tile_x=0, boundary=BOUNDARY_PML, batch=0) -> Config:
    """batch > 1 (VTI): the engine runs up to `batch` shots per launch (Engine.run_shots)."""
    if isinstance(physics, str):
        physics = PHYSICS[physics]
    if isinstance(boundary, str):
        boundary = BOUNDARIES[boundary]
    return Config(physics, nx, ny, nz, dx, dy, dz, nt, dt, fm, wtype, npml, rec_z, int(mute), storage, tile_x,
                  boundary, batch)


class Engine:
    """A model resident on the GPU; run shots against it."""

    def __init__(self, cfg: Config, models: dict, device: int = 0):
        self.cfg = cfg
        n = cfg.nx * cfg.ny * cfg.nz
        self._keep = {}
        ptrs = []
        for name in MODEL_NAMES:
            a = models.get(name)
            if a is not None and name in READS[cfg.physics]:
                a = np.ascontiguousarray(a, dtype=np.float32).reshape(-1)
                if a.size != n:
                    raise ValueError(f"model {name} has {a.size} values, expected {n}")
                self._keep[name] = a
            else:
                a = None
            ptrs.append(_fptr(a))
        h = ctypes.c_void_p()
        _check(lib().a3d_engine_create(ctypes.byref(h), ctypes.byref(cfg), *ptrs, device))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().a3d_engine_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, sx, sy, sz, snap_every=0, snap_skip0=False, with_time=False):
        """Run one shot; returns record[ny, nx, nt] (and snapshots, device ms)."""
        c = self.cfg
        rec = np.zeros((c.ny, c.nx, c.nt), dtype=np.float32)
        nsnap = 0
        if snap_every > 0:
            nsnap = sum(1 for it in range(c.nt) if it % snap_every == 0 and not (snap_skip0 and it == 0))
        snaps = np.zeros((max(nsnap, 1), c.ny, c.nx, c.nz), np.float32) if nsnap else None
        ms = ctypes.c_double(0.0)
        _check(lib().a3d_engine_run(self.h, ctypes.byref(ShotPos(sx, sy, sz)), _fptr(rec), snap_every,
                                    int(snap_skip0), _fptr(snaps), ctypes.byref(ms)))
        out = (rec,)
        if snap_every > 0:
            out += (snaps,)
        if with_time:
            out += (ms.value,)
        return out[0] if len(out) == 1 else out

    def run_shots(self, shots, with_time=False, to_host=True):
        """Multi-shot sweep (engine made with batch >= len(shots)): records
        [k, ny, nx, nt] (None with to_host=False: they stay on the device), and the
        device ms of the time loop with with_time."""
        c = self.cfg
        k = len(shots)
        arr = (ShotPos * max(k, 1))(*[ShotPos(*s) for s in shots])
        recs = np.zeros((k, c.ny, c.nx, c.nt), np.float32) if to_host else None
        ms = ctypes.c_double(0.0)
        _check(lib().a3d_engine_run_shots(self.h, arr, k, _fptr(recs), ctypes.byref(ms)))
        return (recs, ms.value) if with_time else recs

    def record(self, j=0):
        """The record [ny, nx, nt] of shot j of the last run (a3d_engine_copy_record)."""
        c = self.cfg
        rec = np.zeros((c.ny, c.nx, c.nt), np.float32)
        _check(lib().a3d_engine_copy_record(self.h, j, _fptr(rec)))
        return rec

    def run_device(self, sx, sy, sz, rec_dev_ptr=None) -> float:
        """Run one shot leaving the record on the device; returns device ms."""
        ms = ctypes.c_double(0.0)
        _check(lib().a3d_engine_run_device(self.h, ctypes.byref(ShotPos(sx, sy, sz)),
                                           ctypes.c_void_p(rec_dev_ptr), ctypes.byref(ms)))
        return ms.value

    def set_profiling(self, on: bool):
        _check(lib().a3d_engine_set_profiling(self.h, int(on)))

    def kernel_times(self):
        """([ms_vel_or_step, ms_stress], [launches, launches]) summed since profiling was enabled."""
        ms = (ctypes.c_double * 2)()
        n = (ctypes.c_longlong * 2)()
        _check(lib().a3d_engine_kernel_times(self.h, ms, n))
        return [ms[0], ms[1]], [n[0], n[1]]

    def describe(self) -> dict:
        import json
        buf = ctypes.create_string_buffer(2048)
        _check(lib().a3d_engine_describe(self.h, buf, len(buf)))
        return json.loads(buf.value.decode())

    def set_closure(self, params):
        """Install the learned rim's weights (engine created with boundary 'learned')."""
        p = np.ascontiguousarray(params, dtype=np.float32).reshape(-1)
        _check(lib().a3d_engine_set_closure(self.h, _fptr(p), p.size))

    def set_tap(self, steps, off, dev_ptr):
        """After each listed step copy u, v, w, P over [off, nn - off) to device memory."""
        arr = (ctypes.c_int * max(len(steps), 1))(*steps)
        _check(lib().a3d_engine_set_tap(self.h, arr, len(steps), off, ctypes.c_void_p(dev_ptr)))

    def closure_times(self):
        """(ms, launch pairs) of the closure summed since profiling was enabled."""
        ms = ctypes.c_double(0.0)
        n = ctypes.c_longlong(0)
        _check(lib().a3d_engine_closure_times(self.h, ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value

    def record_device_ptr(self) -> int:
        return lib().a3d_engine_record_device(self.h)

    def device_bytes(self) -> int:
        return lib().a3d_engine_device_bytes(self.h)


def forward_host(cfg: Config, models: dict, shots, device: int = 0):
    """One call from host buffers: upload, run every shot, copy the records back."""
    n = cfg.nx * cfg.ny * cfg.nz
    ptrs, keep = [], []
    for name in MODEL_NAMES:
        a = models.get(name)
        if a is not None and name in READS[cfg.physics]:
            a = np.ascontiguousarray(a, dtype=np.float32).reshape(-1)
            assert a.size == n
            keep.append(a)
            ptrs.append(_fptr(a))
        else:
            ptrs.append(_fptr(None))
    arr = (ShotPos * len(shots))(*[ShotPos(*s) for s in shots])
    recs = np.zeros((len(shots), cfg.ny, cfg.nx, cfg.nt), np.float32)
    _check(lib().a3d_forward_host(ctypes.byref(cfg), *ptrs, arr, len(shots), _fptr(recs), device))
    return recs


def run_batch(cfg: Config, models: dict, shots, windows=None, graph: bool = False, device: int = 0):
    """Every shot of a survey in one call (a3d_run_batch).

    windows: None, or one (x0, y0, z0, nx, ny, nz) per shot (nx == 0: whole model).
    Returns (records, ms): records[i] is shot i's [wny][wnx][nt] array, ms[i] the
    device time of its time loop."""
    n = cfg.nx * cfg.ny * cfg.nz
    keep, ptrs = [], []
    for name in MODEL_NAMES:
        a = models.get(name)
        if a is not None and name in READS[cfg.physics]:
            a = np.ascontiguousarray(a, dtype=np.float32).reshape(-1)
            if a.size != n:
                raise ValueError(f"model {name} has {a.size} values, expected {n}")
            keep.append(a)
            ptrs.append(_fptr(a))
        else:
            ptrs.append(_fptr(None))
    pb = Problem(cfg, *ptrs)
    ns = len(shots)
    arr = (ShotPos * max(ns, 1))(*[ShotPos(*s) for s in shots])
    dims = []
    win = None
    if windows is not None:
        if len(windows) != ns:
            raise ValueError("one window per shot")
        win = (Window * max(ns, 1))(*[Window(*w) for w in windows])
        dims = [(w[4], w[3]) if w[3] else (cfg.ny, cfg.nx) for w in windows]
    else:
        dims = [(cfg.ny, cfg.nx)] * ns
    total = sum(a * b for a, b in dims) * cfg.nt
    recs = np.zeros(max(total, 1), np.float32)
    offs = (ctypes.c_size_t * max(ns, 1))()
    ms = (ctypes.c_double * max(ns, 1))()
    opts = Opts(device, win, int(graph), _fptr(recs), offs, ms)
    _check(lib().a3d_run_batch(ctypes.byref(pb), arr, ns, ctypes.byref(opts)))
    out = [recs[offs[i]:offs[i] + dims[i][0] * dims[i][1] * cfg.nt].reshape(dims[i][0], dims[i][1], cfg.nt)
           for i in range(ns)]
    return out, [ms[i] for i in range(ns)]


class Closure:
    """Training object of the learned rim (a3d_closure_*): teacher state pairs of
    nx*ny*nz models on the rim grid (model + 10 cells per face), trained on the GPU."""

    def __init__(self, nx, ny, nz, device: int = 0):
        self.shape = (ny + 2 * CLOSURE_PAD, nx + 2 * CLOSURE_PAD, nz + 2 * CLOSURE_PAD)  # (y, x, z)
        h = ctypes.c_void_p()
        _check(lib().a3d_closure_create(ctypes.byref(h), nx, ny, nz, device))
        self.h = h
        self.n = (nx, ny, nz)

    def close(self):
        if getattr(self, "h", None):
            lib().a3d_closure_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, params):
        p = np.ascontiguousarray(params, dtype=np.float32).reshape(-1)
        _check(lib().a3d_closure_set_params(self.h, _fptr(p), p.size))

    def params(self):
        p = np.zeros(CLOSURE_NPARAM, np.float32)
        _check(lib().a3d_closure_get_params(self.h, _fptr(p), p.size))
        return p

    def add_model(self, vel, rho, dx, dy, dz, dt) -> int:
        n = self.n[0] * self.n[1] * self.n[2]
        v = np.ascontiguousarray(vel, np.float32).reshape(-1)
        r = np.ascontiguousarray(rho, np.float32).reshape(-1)
        if v.size != n or r.size != n:
            raise ValueError("model arrays must hold nx*ny*nz values")
        mid = ctypes.c_int(-1)
        _check(lib().a3d_closure_add_model(self.h, _fptr(v), _fptr(r), dx, dy, dz, dt, ctypes.byref(mid)))
        return mid.value

    def staging(self, nstates) -> int:
        """Device buffer of nstates rim-grid states (4 fields each), owned by the object."""
        p = lib().a3d_closure_staging(self.h, nstates)
        if not p:
            raise A3DError(A3D_E_NOMEM, last_error())
        return p

    def state_floats(self) -> int:
        return 4 * self.shape[0] * self.shape[1] * self.shape[2]

    def add_sample(self, model, state0_ptr, state1_ptr):
        _check(lib().a3d_closure_add_sample(self.h, model, ctypes.c_void_p(state0_ptr), ctypes.c_void_p(state1_ptr)))

    def num_samples(self) -> int:
        return lib().a3d_closure_num_samples(self.h)

    def set_decay(self, decay):
        _check(lib().a3d_closure_set_decay(self.h, decay))

    def train(self, epochs, batch, lr, seed=0):
        loss = np.zeros(epochs, np.float32)
        _check(lib().a3d_closure_train(self.h, epochs, batch, lr, seed, _fptr(loss)))
        return loss

    def eval(self, sample):
        """(correction [4, y, x, z], loss gradient [NPARAM], loss) of one sample."""
        d = np.zeros((4,) + self.shape, np.float32)
        g = np.zeros(CLOSURE_NPARAM, np.float32)
        loss = np.zeros(1, np.float32)
        _check(lib().a3d_closure_eval(self.h, sample, _fptr(d), _fptr(g), _fptr(loss)))
        return d, g, float(loss[0])

    def eval_tc(self, sample):
        """The correction of one sample by the tensor-core kernels ([4, y, x, z])."""
        d = np.zeros((4,) + self.shape, np.float32)
        _check(lib().a3d_closure_eval_tc(self.h, sample, _fptr(d)))
        return d

    def teacher(self, sample):
        """(step(S_t), S_t+1) of one sample, each [4, y, x, z]."""
        x = np.zeros((4,) + self.shape, np.float32)
        t = np.zeros((4,) + self.shape, np.float32)
        _check(lib().a3d_closure_teacher(self.h, sample, _fptr(x), _fptr(t)))
        return x, t
