"""Host-side mirror of the reference's Python interface (readmodel.py), driving
the sm_103a engines.

Same classes, constructor arguments and run() semantics as the reference's
readmodel.py (Model :1-89, ShotReceiver :92-136, FD :139-204, Acoustic3d1order
:208-250, Acoustic3dvti :253-296, Acoustic3d2order :299-339, Acoustic3dtti
:341-386), so scripts written for it (pyAcoustic.py) run unchanged with
``from readmodel import *``.  Differences, all deliberate:

* the libraries load from this package's lib/ directory (absolute path), not
  './lib' relative to the working directory, and a missing library raises;
* the ctypes calls declare argtypes/restype, and a nonzero status from the
  engine raises A3DError instead of passing silently;
* Model.read_model works (the reference swaps struct.unpack's arguments,
  readmodel.py:70) and returns the model as an (nx, ny, nz) array;
* FD.run(..., skip_existing=True) skips shots whose record file already exists
  with the expected size (the reference's disabled "exists, skip" branch,
  readmodel.py:224), so an interrupted survey can resume.
"""
from __future__ import annotations

import ctypes
import os
import struct
from ctypes import c_bool, c_char_p, c_float, c_int

import numpy as np

_LIB_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib")


class A3DError(RuntimeError):
    pass


class Model:
    def __init__(self, nx, ny, nz, dx, dy, dz, vel_file=None, rho_file=None, delta_file=None,
                 epsilon_file=None, theta_file=None, psi_file=None):
        self.nx, self.ny, self.nz = nx, ny, nz
        self.dx, self.dy, self.dz = dx, dy, dz
        self.rho_file = rho_file
        self.vel_file = vel_file
        self.delta_file = delta_file
        self.epsilon_file = epsilon_file
        self.theta_file = theta_file
        self.psi_file = psi_file
        self.shape = (self.nx, self.ny, self.nz)

    def write_model(self, filename, value):
        """Homogeneous model file: nx*ny*nz float32 copies of value (readmodel.py:20-29)."""
        if filename is None:
            print(filename, "cannot be None")
            raise NameError
        np.full(self.nx * self.ny * self.nz, value, dtype=np.float32).tofile(filename)

    def write_rho(self, value):
        self.write_model(self.rho_file, value)

    def write_vel(self, value):
        self.write_model(self.vel_file, value)

    def write_epsilon(self, value):
        self.write_model(self.epsilon_file, value)

    def write_delta(self, value):
        self.write_model(self.delta_file, value)

    def write_theta(self, value):
        self.write_model(self.theta_file, value)

    def write_psi(self, value):
        self.write_model(self.psi_file, value)

    def generate_model(self, vel=3000, rho=1200, epsilon=0.0, delta=0.0, theta=0.0, psi=0.0):
        """As readmodel.py:49-59: epsilon..psi files are written only when nonzero."""
        self.write_vel(vel)
        self.write_rho(rho)
        if epsilon != 0.0:
            self.write_epsilon(epsilon)
        if delta != 0.0:
            self.write_delta(delta)
        if theta != 0.0:
            self.write_theta(theta)
        if psi != 0.0:
            self.write_psi(psi)

    def read_model(self, filename):
        """Model file as an (nx, ny, nz) float32 array (file order: z fastest, x, y)."""
        a = np.fromfile(filename, dtype=np.float32)
        if a.size != self.nx * self.ny * self.nz:
            raise ValueError(f"{filename}: {a.size} values, expected {self.nx * self.ny * self.nz}")
        return np.ascontiguousarray(a.reshape(self.ny, self.nx, self.nz).transpose(1, 0, 2))

    def __str__(self):
        res = "*" * 30 + "\n"
        res += "the size of model is:\n"
        res += "nx, ny, nz = {}, {}, {}\n".format(self.nx, self.ny, self.nz)
        res += "dx, dy, dz = {}, {}, {}\n".format(self.dx, self.dy, self.dz)
        res += "*" * 30 + "\n"
        res += "velocity file : " + str(self.vel_file) + "\n"
        if self.rho_file:
            res += "density file : " + self.rho_file + "\n"
        if self.delta_file:
            res += "delta file : " + self.delta_file + "\n"
        if self.epsilon_file:
            res += "epsilon file: " + self.epsilon_file + "\n"
        res += "*" * 30 + "\n"
        return res


class ShotReceiver:
    def __init__(self, sxbeg, sybeg, szbeg, jsx, jsy, jsz, sxend, syend, szend, dgx, dgy, dgt, shotfolder):
        self.sxbeg, self.sybeg, self.szbeg = sxbeg, sybeg, szbeg
        self.jsx, self.jsy, self.jsz = jsx, jsy, jsz
        self.sxend, self.syend, self.szend = sxend, syend, szend
        self.shotfile = shotfolder
        self.shotlist = self.generateShotList()
        self.nshot = len(self.shotlist)
        self.nodetask = self.allocateNode()
        self.receiver_dx = dgx
        self.receiver_dy = dgy
        self.receiver_dt = dgt

    def generateShotList(self):
        """x outermost, then y, then z (readmodel.py:112-119)."""
        shotlist = []
        for isx in range(self.sxbeg, self.sxend + 1, self.jsx):
            for isy in range(self.sybeg, self.syend + 1, self.jsy):
                for isz in range(self.szbeg, self.szend + 1, self.jsz):
                    shotlist.append((isx, isy, isz, self.jsx, self.jsy, self.jsz))
        self.shotlist = shotlist
        return shotlist

    def allocateNode(self, nnode=1):
        """Round-robin split of the shots over nnode hosts (readmodel.py:121-126)."""
        self.nodetask = [self.shotlist[i::nnode] for i in range(nnode)]
        return self.nodetask

    def __str__(self):
        res = "*" * 30 + "\n"
        res += "the shot begin: {}, {}, {}\n".format(self.sxbeg, self.sybeg, self.szbeg)
        res += "the shot inverval: {}, {}, {}\n".format(self.jsx, self.jsy, self.jsz)
        res += "the geophone interval: {}, {}\n".format(self.receiver_dx, self.receiver_dy)
        res += "the geophone sampling time: {}\n".format(self.receiver_dt)
        res += "shot shotfolder is " + self.shotfile + "\n"
        res += "*" * 30 + "\n"
        return res


_SIGS = {
    "cuda_3dfd": [c_char_p] * 3 + [c_int] * 5 + [c_float] * 3 + [c_int] * 6 + [c_float] * 3 +
                 [c_int, c_int, c_float, c_float, c_bool, c_bool, c_int, c_int],
    "cuda_3dfd_1order": [c_char_p] * 4 + [c_int] * 5 + [c_float] * 3 + [c_int] * 6 + [c_float] * 3 +
                        [c_int, c_float, c_int, c_float, c_bool, c_bool, c_int, c_int],
    "cuda_3dfd_vti": [c_char_p] * 6 + [c_int] * 5 + [c_float] * 3 + [c_int] * 6 + [c_float] * 3 +
                     [c_int, c_float, c_float, c_bool, c_bool, c_int, c_int],
    "cuda_3dfd_tti": [c_char_p] * 8 + [c_int] * 5 + [c_float] * 3 + [c_int] * 6 + [c_float] * 3 +
                     [c_int, c_float, c_float, c_bool, c_bool, c_int, c_int],
}


def _load(libname, symbol):
    path = os.path.join(_LIB_DIR, libname)
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: run acoustic3d-fd_gb300/build.py")
    fn = getattr(ctypes.cdll.LoadLibrary(path), symbol)
    fn.argtypes = _SIGS[symbol]
    fn.restype = c_int
    return fn


def _s(x):
    return c_char_p(bytes(x if x is not None else "", "utf-8"))


class FD:
    libname = None
    symbol = None
    physics = None  # engine of the batched path: "2o", "iso", "vti", "tti"

    def __init__(self, model, sg, nt, dt, fpeak, snap_folder, snap_interval, wtype=1, device_i=0,
                 savesnap=False, nodei=0, cut_directwave=False):
        self.model = model
        self.nt = nt
        self.dt = dt
        self.sg = sg
        self.fpeak = fpeak
        self.snap_folder = snap_folder
        self.snap_interval = snap_interval
        self.kernel = None
        self.savesnap = savesnap
        self.nodei = nodei
        self.cut_directwave = cut_directwave
        self.wtype = wtype
        assert self.sg.receiver_dx % self.model.dx == 0
        assert self.sg.receiver_dy % self.model.dy == 0
        assert self.sg.receiver_dt % self.dt == 0

    def __str__(self):
        res = "the Model Property: \n" + str(self.model)
        res += "the Receiver and Shot setting:\n" + str(self.sg)
        res += "the dominant frequency: {}\n".format(self.fpeak)
        res += "nt : {}, dt : {}\n".format(self.nt, self.dt)
        res += "save snapshot : {}\n".format(self.savesnap)
        if self.savesnap:
            res += "snap interval : {}\n".format(self.snap_interval)
            res += "snap folder : {}\n".format(self.snap_folder)
        res += "cut direct wave : {}\n".format(self.cut_directwave)
        return res

    def load_kernel(self):
        self.kernel = _load(self.libname, self.symbol)

    def available_GPU(self):
        """Device with the largest free/total memory ratio (readmodel.py:173-184)."""
        import subprocess
        total = subprocess.getoutput("nvidia-smi --query-gpu=memory.total --format=csv,noheader,nounits")
        free = subprocess.getoutput("nvidia-smi --query-gpu=memory.free --format=csv,noheader,nounits")
        t = np.array([float(x) for x in total.split()])
        f = np.array([float(x) for x in free.split()])
        return int(np.argmax(f / t))

    def shot_name(self, ishot):
        return self.sg.shotfile + "{0}.{1}.bin".format(str(ishot[0]), str(ishot[1]))

    def record_bytes(self):
        jx = int(self.sg.receiver_dx / self.model.dx)
        jy = int(self.sg.receiver_dy / self.model.dy)
        jt = int(np.float32(self.sg.receiver_dt) / np.float32(self.dt))
        nx, ny, nt = self.model.nx, self.model.ny, self.nt
        return 4 * len(range(0, nx, jx)) * len(range(0, ny, jy)) * len(range(0, nt, jt))

    def run(self, ishot, device, skip_existing=False):
        self.load_kernel()
        if device is None:
            device = self.available_GPU()
        print("device: {}, shot: ".format(device), ishot)
        shotname = self.shot_name(ishot)
        if skip_existing and os.path.exists(shotname) and os.path.getsize(shotname) == self.record_bytes():
            print(shotname + " exists, skip")
            return 0
        rc = self.kernel(*self._args(ishot, shotname, device))
        if rc != 0:
            raise A3DError(f"{self.symbol} returned status {rc} for shot {ishot}")
        return rc

    def _geometry(self, ishot):
        m, sg = self.model, self.sg
        return [c_int(0), c_int(1), c_int(m.nx), c_int(m.ny), c_int(m.nz), c_float(m.dx), c_float(m.dy),
                c_float(m.dz), c_int(ishot[0]), c_int(ishot[1]), c_int(ishot[2]), c_int(ishot[3]),
                c_int(ishot[4]), c_int(ishot[5]), c_float(sg.receiver_dx), c_float(sg.receiver_dy),
                c_float(sg.receiver_dt)]

    def parallel_run(self, skip_existing=False):
        """One worker process per GPU, shots of this node handed out in order
        (readmodel.py:186-204): replicas, no communication between shots."""
        from multiprocessing import get_context
        import subprocess
        n_dev = int(subprocess.getoutput("nvidia-smi -L | grep GPU | wc -l") or 1)
        tasks = list(self.sg.nodetask[self.nodei])
        ctx = get_context("spawn")
        with ctx.Pool(n_dev) as pool:
            res = [pool.apply_async(self.run, (t, i % n_dev, skip_existing)) for i, t in enumerate(tasks)]
            for r in res:
                r.get()


    # ---- batched path: one process per GPU feeding a3d_run_batch (replaces the
    # process-per-shot pool and the nvidia-smi polling of readmodel.py:173-204)
    _MODEL_FILES = {"vel": "vel_file", "rho": "rho_file", "eps": "epsilon_file", "del": "delta_file",
                    "theta": "theta_file", "phi": "psi_file"}
    _READS = {"2o": ("vel",), "iso": ("vel", "rho"), "vti": ("vel", "rho", "eps", "del"),
              "tti": ("vel", "eps", "del", "theta", "phi")}

    def engine_config(self):
        """The engine configuration the legacy entry point of this class builds."""
        import a3d
        m = self.model
        return a3d.make_config(self.physics, m.nx, m.ny, m.nz, dx=m.dx, dy=m.dy, dz=m.dz, nt=self.nt, dt=self.dt,
                               fm=self.fpeak, wtype=self.wtype if self.physics == "iso" else 1, npml=0,
                               rec_z=-1, mute=bool(self.cut_directwave) and self.physics != "2o")

    def read_models(self):
        m = self.model
        n = m.nx * m.ny * m.nz
        out = {}
        for k in self._READS[self.physics]:
            a = np.fromfile(getattr(m, self._MODEL_FILES[k]), dtype=np.float32, count=n)
            if a.size != n:
                raise A3DError(f"model file for {k} holds {a.size} of {n} floats")
            out[k] = a
        return out

    def write_record(self, shotname, rec):
        """The legacy writer's layout: iy (step dgy/dy), ix (step dgx/dx), it (step dgt/dt)."""
        jx = int(self.sg.receiver_dx / self.model.dx)
        jy = int(self.sg.receiver_dy / self.model.dy)
        jt = int(np.float32(self.sg.receiver_dt) / np.float32(self.dt))
        np.ascontiguousarray(rec[::jy, ::jx, ::jt], dtype=np.float32).tofile(shotname)

    _STORAGE = {"fp32": 0, "bf16": 1, "fp16": 2, "fp16v": 4}

    def _survey_worker(self, tasks, device, graph, batch=0, chunk=4, storage="fp32"):
        """Runs the tasks on one device, `chunk` shots per a3d_run_batch call (the
        multi-shot batch size for VTI when batch > 1); a writer thread writes each
        call's record files while the next call runs on the GPU (the call releases
        the interpreter lock), so file output overlaps compute and the host holds
        at most two calls' records."""
        import queue
        import threading
        import a3d
        if not tasks:
            return 0
        cfg = self.engine_config()
        cfg.batch = batch if (batch > 1 and self.physics == "vti") else 0
        cfg.storage = self._STORAGE[storage]
        models = self.read_models()
        step = max(cfg.batch, chunk, 1)
        q = queue.Queue(maxsize=1)
        failed = []

        def writer():
            while True:
                item = q.get()
                if item is None:
                    return
                if failed:
                    continue
                try:
                    for t, rec in item:
                        self.write_record(self.shot_name(t), rec)
                except Exception as exc:  # reported after the GPU work stops
                    failed.append(exc)

        th = threading.Thread(target=writer, daemon=True)
        th.start()
        try:
            for i in range(0, len(tasks), step):
                part = tasks[i:i + step]
                recs, _ = a3d.run_batch(cfg, models, [tuple(t[:3]) for t in part], graph=graph, device=device)
                if failed:
                    break
                q.put(list(zip(part, recs)))
        finally:
            q.put(None)
            th.join()
        if failed:
            raise failed[0]
        return len(tasks)

    def survey(self, devices=(0,), skip_existing=False, graph=True, batch=0, storage="fp32"):
        """Every shot of this node through the batched entry point: one worker process
        per device, each with its round-robin share of the shots (as allocateNode splits
        nodes, readmodel.py:121-126) in a3d_run_batch calls, records written in the
        legacy layout while the next shots run.  batch > 1 (VTI): shots advance that
        many at a time in multi-shot sweeps.  storage: "fp32" (the legacy entry points'
        arithmetic), or "bf16" / "fp16" (1st-order engines) / "fp16v" (VTI, TTI) for
        the reduced-precision wavefield forms.  With skip_existing, complete record
        files are kept (resume).  Snapshots are not taken on this path (run() takes
        them)."""
        if storage not in self._STORAGE:
            raise A3DError(f"storage {storage!r} is not one of {sorted(self._STORAGE)}")
        tasks = [t for t in self.sg.nodetask[self.nodei]
                 if not (skip_existing and os.path.exists(self.shot_name(t)) and
                         os.path.getsize(self.shot_name(t)) == self.record_bytes())]
        devices = list(devices)
        if len(devices) == 1:
            return self._survey_worker(tasks, devices[0], graph, batch, 4, storage)
        from multiprocessing import get_context
        ctx = get_context("spawn")
        with ctx.Pool(len(devices)) as pool:
            res = [pool.apply_async(self._survey_worker, (tasks[k::len(devices)], d, graph, batch, 4, storage))
                   for k, d in enumerate(devices)]
            return sum(r.get() for r in res)


class Acoustic3d1order(FD):
    libname, symbol = "acoustic1order.so", "cuda_3dfd_1order"
    physics = "iso"

    def _args(self, ishot, shotname, device):
        m = self.model
        return ([_s(m.vel_file), _s(m.rho_file), _s(self.snap_folder), _s(shotname)] + self._geometry(ishot) +
                [c_int(self.nt), c_float(self.dt), c_int(self.wtype), c_float(self.fpeak), c_bool(self.savesnap),
                 c_bool(self.cut_directwave), c_int(self.snap_interval), c_int(device)])

    def __str__(self):
        return "Stencil Acoustic 3D first order\n" + "*" * 30 + "\n" + super().__str__()


class Acoustic3dvti(FD):
    libname, symbol = "acoustic1vti.so", "cuda_3dfd_vti"
    physics = "vti"

    def _args(self, ishot, shotname, device):
        m = self.model
        return ([_s(m.vel_file), _s(m.rho_file), _s(m.epsilon_file), _s(m.delta_file), _s(self.snap_folder),
                 _s(shotname)] + self._geometry(ishot) +
                [c_int(self.nt), c_float(self.dt), c_float(self.fpeak), c_bool(self.savesnap),
                 c_bool(self.cut_directwave), c_int(self.snap_interval), c_int(device)])

    def __str__(self):
        return "Stencil Acoustic vti 3D \n" + "*" * 30 + "\n" + super().__str__()


class Acoustic3d2order(FD):
    libname, symbol = "acoustic2order.so", "cuda_3dfd"
    physics = "2o"

    def _args(self, ishot, shotname, device):
        m = self.model
        # the reference's caller passes kt=300 and swaps the last two flags (readmodel.py:335-338);
        # the engine ignores all three, as the reference does
        return ([_s(m.vel_file), _s(self.snap_folder), _s(shotname)] + self._geometry(ishot) +
                [c_int(self.nt), c_int(300), c_float(self.dt), c_float(self.fpeak), c_bool(self.savesnap),
                 c_bool(self.cut_directwave), c_int(self.snap_interval), c_int(device)])

    def __str__(self):
        return "Stencil Acoustic 3D second order\n" + "*" * 30 + "\n" + super().__str__()


class Acoustic3dtti(FD):
    libname, symbol = "acoustic1tti.so", "cuda_3dfd_tti"
    physics = "tti"

    def _args(self, ishot, shotname, device):
        m = self.model
        return ([_s(m.vel_file), _s(m.rho_file), _s(m.epsilon_file), _s(m.delta_file), _s(m.theta_file),
                 _s(m.psi_file), _s(self.snap_folder), _s(shotname)] + self._geometry(ishot) +
                [c_int(self.nt), c_float(self.dt), c_float(self.fpeak), c_bool(self.savesnap),
                 c_bool(self.cut_directwave), c_int(self.snap_interval), c_int(device)])

    def __str__(self):
        return "Stencil Acoustic tti 3D \n" + "*" * 30 + "\n" + super().__str__()


__all__ = ["Model", "ShotReceiver", "FD", "Acoustic3d1order", "Acoustic3dvti", "Acoustic3d2order",
           "Acoustic3dtti", "A3DError"]
