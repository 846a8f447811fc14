"""The reference's own Python caller, unmodified, against this build's libraries.

readmodel.py's FD subclasses (readmodel.py:207-386) load ./lib/<name>.so relative
to the working directory and call the drop-in entry points through ctypes with no
argtypes or restype.  This test imports that file from the reference checkout
(it is read, not copied: the directory named by A3D_REFERENCE, else a checkout
named "reference" beside this repository; skipped where there is none), runs each
class's run() in a temporary directory whose ./lib holds this build's four
libraries, and checks, through the libraries' call trace (A3D_LEGACY_TRACE: one
JSON line per call with every argument as received, written before any other
work), that every argument arrives as the caller meant it.  On a machine without
a GPU the calls then return A3D_E_CUDA, which readmodel.py ignores; the GPU-side
results of the same calls are checked file by file in tests/test_gpu_dropin.py.
"""
import importlib.util
import json
import os

import numpy as np
import pytest

from conftest import PKG, ROOT

REF = os.environ.get("A3D_REFERENCE") or os.path.join(os.path.dirname(ROOT), "reference")
RM_PATH = os.path.join(REF, "readmodel.py")


def _readmodel():
    if not os.path.exists(RM_PATH):
        pytest.skip(f"no reference checkout with readmodel.py at {REF}")
    spec = importlib.util.spec_from_file_location("reference_readmodel", RM_PATH)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture()
def workdir(engine_lib, tmp_path, monkeypatch):
    lib = tmp_path / "lib"
    lib.mkdir()
    for name in ("acoustic2order.so", "acoustic1order.so", "acoustic1vti.so", "acoustic1tti.so"):
        os.symlink(os.path.join(PKG, "lib", name), lib / name)
    trace = tmp_path / "trace.jsonl"
    monkeypatch.setenv("A3D_LEGACY_TRACE", str(trace))
    monkeypatch.chdir(tmp_path)
    return tmp_path, trace


def _calls(trace):
    with open(trace) as f:
        return [json.loads(line) for line in f]


def _setup(RM, d):
    nx, ny, nz = 12, 10, 8
    m = RM.Model(nx, ny, nz, 10.0, 10.0, 10.0, vel_file=str(d / "vel.bin"), rho_file=str(d / "rho.bin"),
                 delta_file=str(d / "del.bin"), epsilon_file=str(d / "eps.bin"),
                 theta_file=str(d / "theta.bin"), psi_file=str(d / "psi.bin"))
    m.generate_model(vel=2500.0, rho=2000.0, epsilon=0.2, delta=0.1, theta=0.3, psi=0.4)
    sg = RM.ShotReceiver(5, 4, 3, 2, 1, 1, 7, 4, 3, 20.0, 10.0, 0.002, str(d / "shot_"))
    return m, sg


def _check_geometry(c, m, sg, shot, d):
    assert (c["nx"], c["ny"], c["nz"]) == (m.nx, m.ny, m.nz)
    assert (c["dx"], c["dy"], c["dz"]) == (10.0, 10.0, 10.0)
    assert (c["sxbeg"], c["sybeg"], c["szbeg"], c["jsx"], c["jsy"], c["jsz"]) == tuple(shot)
    assert (c["is"], c["ns"]) == (0, 1)
    assert c["dgx"] == 20.0 and c["dgy"] == 10.0 and c["dgt"] == np.float32(0.002)
    assert c["FNshot"] == str(d / "shot_") + f"{shot[0]}.{shot[1]}.bin"


def test_first_order_vti_tti_callers(workdir):
    RM = _readmodel()
    d, trace = workdir
    m, sg = _setup(RM, d)
    shot = sg.shotlist[1]
    kw = dict(nt=40, dt=0.001, fpeak=25.0, snap_folder=str(d / "snap_"), snap_interval=10, wtype=3,
              savesnap=True, cut_directwave=True)
    RM.Acoustic3d1order(m, sg, **kw).run(shot, 0)
    RM.Acoustic3dvti(m, sg, **kw).run(shot, 0)
    RM.Acoustic3dtti(m, sg, **kw).run(shot, 0)
    calls = _calls(trace)
    assert [c["entry"] for c in calls] == ["cuda_3dfd_1order", "cuda_3dfd_vti", "cuda_3dfd_tti"]
    for c in calls:
        _check_geometry(c, m, sg, shot, d)
        assert c["nt"] == 40 and c["dt"] == np.float32(0.001) and c["fm"] == 25.0
        assert c["show_snapshot"] is True and c["cut_directwave"] is True
        assert c["snap_interval"] == 10 and c["cudaDevicei"] == 0
        assert c["FNvel"] == m.vel_file and c["FNsnap"] == str(d / "snap_")
    assert calls[0]["FNrho"] == m.rho_file and calls[0]["wtype"] == 3
    assert calls[1]["FNepsilon"] == m.epsilon_file and calls[1]["FNdelta"] == m.delta_file
    assert calls[2]["FNtheta"] == m.theta_file and calls[2]["FNpsi"] == m.psi_file


def test_second_order_caller_swapped_arguments(workdir):
    """Acoustic3d2order passes snap_interval where cut_directwave belongs and the
    other way round (readmodel.py:335-338) and kt = 300; the library, like the
    reference, uses none of the three, and every other argument arrives intact."""
    RM = _readmodel()
    d, trace = workdir
    m, sg = _setup(RM, d)
    shot = sg.shotlist[0]
    RM.Acoustic3d2order(m, sg, nt=30, dt=0.001, fpeak=30.0, snap_folder=str(d / "snap_"), snap_interval=10,
                        savesnap=False, cut_directwave=False).run(shot, 0)
    (c,) = _calls(trace)
    assert c["entry"] == "cuda_3dfd"
    _check_geometry(c, m, sg, shot, d)
    assert c["nt"] == 30 and c["kt"] == 300 and c["dt"] == np.float32(0.001) and c["fm"] == 30.0
    assert c["show_snapshot"] is False and c["cudaDevicei"] == 0
