"""Drop-in entry points: the four legacy symbols called the way readmodel.py calls
them (ctypes, no argtypes/restype; readmodel.py:228-244, 278-296, 324-339, 366-385),
checked file by file against the engine's in-memory API.

Record files: the reference's byte layout (iy, ix, it loops with receiver/time
decimation, offset is*nt*nx*ny*4; ..iso..:590-598).  Snapshot files: names and
contents per engine (2O every 500 steps, iso "ishot_<is>it_<it>", VTI/TTI
"ishot_<is>_it_<it>", TTI every 100 steps regardless of show_snapshot).
"""
import ctypes
import os
from ctypes import c_bool, c_char_p, c_float, c_int

import numpy as np
import pytest

from conftest import PKG
from helpers import decimate, make_models

pytestmark = pytest.mark.gpu


def _b(s):
    return c_char_p(bytes(s, "utf-8"))


def _write(models, d):
    paths = {}
    for k, a in models.items():
        p = os.path.join(d, f"{k}.bin")
        a.tofile(p)
        paths[k] = p
    return paths


def _engine_record(eng, models, nx, ny, nz, nt, dt, fm, shot, mute=False, wtype=1, snap_every=0,
                   snap_skip0=False):
    import a3d
    cfg = a3d.make_config(eng, nx, ny, nz, nt=nt, dt=dt, fm=fm, wtype=wtype, mute=mute)
    e = a3d.Engine(cfg, models)
    out = e.run(*shot, snap_every=snap_every, snap_skip0=snap_skip0)
    e.close()
    return out


def test_acoustic1order_file_output(engine_lib, tmp_path):
    nx, ny, nz, nt, dt, fm = 20, 18, 16, 120, 1e-3, 25.0
    m = make_models("iso", nx, ny, nz, seed=31)
    p = _write(m, tmp_path)
    snapdir = str(tmp_path) + "/snap_"
    shotfile = str(tmp_path / "9.8.bin")
    lib = ctypes.cdll.LoadLibrary(os.path.join(PKG, "lib", "acoustic1order.so"))
    rc = lib.cuda_3dfd_1order(_b(p["vel"]), _b(p["rho"]), _b(snapdir), _b(shotfile), c_int(0), c_int(1),
                              c_int(nx), c_int(ny), c_int(nz), c_float(10), c_float(10), c_float(10),
                              c_int(9), c_int(8), c_int(4), c_int(10), c_int(10), c_int(1),
                              c_float(20.0), c_float(10.0), c_float(2e-3), c_int(nt), c_float(dt), c_int(1),
                              c_float(fm), c_bool(True), c_bool(True), c_int(50), c_int(0))
    assert rc == 0
    rec, snaps = _engine_record("iso", m, nx, ny, nz, nt, dt, fm, (9, 8, 4), mute=True, snap_every=50)
    got = np.fromfile(shotfile, np.float32)
    assert np.array_equal(got, decimate(rec, 2, 1, 2))
    for k, it in enumerate((0, 50, 100)):
        f = f"{snapdir}ishot_0it_{it}.bin"
        assert os.path.exists(f), f
        assert np.array_equal(np.fromfile(f, np.float32), snaps[k].ravel())


def test_acoustic1order_multishot_offsets(engine_lib, tmp_path):
    """ns > 1: shots along x at sxbeg + is*jsx, record is at byte offset is*nt*nx*ny*4."""
    nx, ny, nz, nt, dt, fm = 16, 14, 12, 60, 1e-3, 30.0
    m = make_models("iso", nx, ny, nz, seed=32)
    p = _write(m, tmp_path)
    shotfile = str(tmp_path / "line.bin")
    lib = ctypes.cdll.LoadLibrary(os.path.join(PKG, "lib", "acoustic1order.so"))
    rc = lib.cuda_3dfd_1order(_b(p["vel"]), _b(p["rho"]), _b(str(tmp_path) + "/"), _b(shotfile), c_int(0),
                              c_int(3), c_int(nx), c_int(ny), c_int(nz), c_float(10), c_float(10), c_float(10),
                              c_int(2), c_int(7), c_int(3), c_int(5), c_int(1), c_int(1),
                              c_float(10.0), c_float(10.0), c_float(1e-3), c_int(nt), c_float(dt), c_int(2),
                              c_float(fm), c_bool(False), c_bool(False), c_int(0), c_int(0))
    assert rc == 0
    got = np.fromfile(shotfile, np.float32)
    n = nt * nx * ny
    assert got.size == 3 * n
    for k in range(3):
        rec = _engine_record("iso", m, nx, ny, nz, nt, dt, fm, (2 + 5 * k, 7, 3), wtype=2)
        assert np.array_equal(got[k * n:(k + 1) * n], rec.ravel())


def test_acoustic2order_swapped_arguments(engine_lib, tmp_path):
    """readmodel.py passes snap_interval and cut_directwave swapped; both are ignored,
    snapshots every 500 steps, receivers at model depth 1, no mute."""
    nx, ny, nz, nt, dt, fm = 16, 16, 16, 510, 1e-3, 25.0
    m = make_models("2o", nx, ny, nz, seed=33)
    p = _write(m, tmp_path)
    snapdir = str(tmp_path) + "/s_"
    shotfile = str(tmp_path / "8.8.bin")
    lib = ctypes.cdll.LoadLibrary(os.path.join(PKG, "lib", "acoustic2order.so"))
    rc = lib.cuda_3dfd(_b(p["vel"]), _b(snapdir), _b(shotfile), c_int(0), c_int(1), c_int(nx), c_int(ny),
                       c_int(nz), c_float(10), c_float(10), c_float(10), c_int(8), c_int(8), c_int(5),
                       c_int(10), c_int(10), c_int(1), c_float(10.0), c_float(10.0), c_float(1e-3),
                       c_int(nt), c_int(300), c_float(dt), c_float(fm), c_bool(True),
                       c_int(100), c_bool(True), c_int(0))
    assert rc == 0
    rec, snaps = _engine_record("2o", m, nx, ny, nz, nt, dt, fm, (8, 8, 5), snap_every=500)
    assert np.array_equal(np.fromfile(shotfile, np.float32), rec.ravel())
    for k, it in enumerate((0, 500)):
        assert np.array_equal(np.fromfile(f"{snapdir}ishot_0_it_{it}.bin", np.float32), snaps[k].ravel())
    assert not os.path.exists(f"{snapdir}ishot_0_it_100.bin")


def test_acoustic1vti_and_tti_files(engine_lib, tmp_path):
    nx, ny, nz, nt, dt, fm = 18, 16, 14, 210, 1e-3, 25.0
    for eng, libname in (("vti", "acoustic1vti.so"), ("tti", "acoustic1tti.so")):
        m = make_models(eng, nx, ny, nz, seed=34)
        d = tmp_path / eng
        d.mkdir()
        p = _write(m, d)
        snap = str(d) + "/"
        shotfile = str(d / "shot.bin")
        lib = ctypes.cdll.LoadLibrary(os.path.join(PKG, "lib", libname))
        common = [c_int(0), c_int(1), c_int(nx), c_int(ny), c_int(nz), c_float(10), c_float(10), c_float(10),
                  c_int(8), c_int(7), c_int(3), c_int(10), c_int(10), c_int(1), c_float(10.0), c_float(10.0),
                  c_float(1e-3), c_int(nt), c_float(dt), c_float(fm)]
        if eng == "vti":
            rc = lib.cuda_3dfd_vti(_b(p["vel"]), _b(p["rho"]), _b(p["eps"]), _b(p["del"]), _b(snap),
                                   _b(shotfile), *common, c_bool(True), c_bool(False), c_int(70), c_int(0))
            rec, snaps = _engine_record(eng, m, nx, ny, nz, nt, dt, fm, (8, 7, 3), snap_every=70)
            its = (0, 70, 140)
        else:
            rc = lib.cuda_3dfd_tti(_b(p["vel"]), _b("/nonexistent"), _b(p["eps"]), _b(p["del"]),
                                   _b(p["theta"]), _b(p["phi"]), _b(snap), _b(shotfile), *common,
                                   c_bool(False), c_bool(False), c_int(70), c_int(0))
            rec, snaps = _engine_record(eng, m, nx, ny, nz, nt, dt, fm, (8, 7, 3), snap_every=100,
                                        snap_skip0=True)
            its = (100, 200)
        assert rc == 0
        assert np.array_equal(np.fromfile(shotfile, np.float32), rec.ravel())
        for k, it in enumerate(its):
            assert np.array_equal(np.fromfile(f"{snap}ishot_0_it_{it}.bin", np.float32), snaps[k].ravel())


def test_missing_model_file_is_an_error_not_a_crash(engine_lib, tmp_path):
    lib = ctypes.cdll.LoadLibrary(os.path.join(PKG, "lib", "acoustic1order.so"))
    lib.cuda_3dfd_1order.restype = c_int
    rc = lib.cuda_3dfd_1order(_b(str(tmp_path / "nope.bin")), _b(str(tmp_path / "nope2.bin")),
                              _b(str(tmp_path) + "/"), _b(str(tmp_path / "s.bin")), c_int(0), c_int(1),
                              c_int(8), c_int(8), c_int(8), c_float(10), c_float(10), c_float(10),
                              c_int(4), c_int(4), c_int(2), c_int(1), c_int(1), c_int(1),
                              c_float(10.0), c_float(10.0), c_float(1e-3), c_int(10), c_float(1e-3), c_int(1),
                              c_float(20.0), c_bool(False), c_bool(False), c_int(1), c_int(0))
    assert rc == 2  # A3D_E_IO


def test_tti_unwritable_shot_file_returns_1(engine_lib, tmp_path):
    lib = ctypes.cdll.LoadLibrary(os.path.join(PKG, "lib", "acoustic1tti.so"))
    lib.cuda_3dfd_tti.restype = c_int
    bad = _b(str(tmp_path / "no_such_dir" / "s.bin"))
    args = [_b("x")] * 7 + [bad, c_int(0), c_int(1), c_int(8), c_int(8), c_int(8), c_float(10), c_float(10),
                            c_float(10), c_int(4), c_int(4), c_int(2), c_int(1), c_int(1), c_int(1),
                            c_float(10.0), c_float(10.0), c_float(1e-3), c_int(10), c_float(1e-3),
                            c_float(20.0), c_bool(False), c_bool(False), c_int(1), c_int(0)]
    assert lib.cuda_3dfd_tti(*args) == 1
