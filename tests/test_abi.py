"""CPU checks of the C ABI: the libraries build, load, and export every symbol
include/acoustic3d.h declares; argument validation runs before any GPU work."""
import ctypes
import os
import re

import pytest

from conftest import PKG, ROOT

HEADER = os.path.join(ROOT, "include", "acoustic3d.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?(?:int|float\s*\*|size_t|char\s*\*|void)\s+\**(\w+)\s*\(",
                                 src, flags=re.M)))


def test_header_declares_entry_points():
    names = declared_functions()
    for need in ("cuda_3dfd", "cuda_3dfd_1order", "cuda_3dfd_vti", "cuda_3dfd_tti",
                 "a3d_engine_create", "a3d_engine_run", "a3d_engine_destroy", "a3d_forward_host"):
        assert need in names


@pytest.mark.parametrize("libname", ["libacoustic3d.so", "acoustic2order.so", "acoustic1order.so",
                                     "acoustic1vti.so", "acoustic1tti.so"])
def test_library_exports_every_declared_symbol(engine_lib, libname):
    lib = ctypes.CDLL(os.path.join(PKG, "lib", libname))
    for name in declared_functions():
        assert hasattr(lib, name), f"{libname} does not export {name}"


def test_invalid_config_rejected_without_gpu(engine_lib):
    import a3d
    cfg = a3d.make_config("iso", 0, 10, 10)  # nx = 0
    h = ctypes.c_void_p()
    rc = a3d.lib().a3d_engine_create(ctypes.byref(h), ctypes.byref(cfg), *[a3d._fptr(None)] * 6, 0)
    assert rc == a3d.A3D_E_ARG
    assert "must be positive" in a3d.last_error()


def test_half_storage_only_for_first_order_engines(engine_lib):
    """bfloat16 / float16 storage is built for the isotropic, VTI and TTI engines; the
    2nd-order engine refuses it."""
    import a3d
    for phys in ("2o",):
        cfg = a3d.make_config(phys, 10, 10, 10, storage=a3d.BF16)
        h = ctypes.c_void_p()
        rc = a3d.lib().a3d_engine_create(ctypes.byref(h), ctypes.byref(cfg), *[a3d._fptr(None)] * 6, 0)
        assert rc == a3d.A3D_E_UNSUPPORTED


def test_mixed_storage_only_for_vti_and_tti(engine_lib):
    """FP16V (float16 u, v, w, float P, Q) is built for the VTI and TTI engines only."""
    import a3d
    for phys in ("2o", "iso"):
        cfg = a3d.make_config(phys, 10, 10, 10, storage=a3d.FP16V)
        h = ctypes.c_void_p()
        rc = a3d.lib().a3d_engine_create(ctypes.byref(h), ctypes.byref(cfg), *[a3d._fptr(None)] * 6, 0)
        assert rc == a3d.A3D_E_UNSUPPORTED, phys


def test_unsupported_storage_rejected(engine_lib):
    import a3d
    cfg = a3d.make_config("iso", 10, 10, 10, storage=7)
    h = ctypes.c_void_p()
    rc = a3d.lib().a3d_engine_create(ctypes.byref(h), ctypes.byref(cfg), *[a3d._fptr(None)] * 6, 0)
    assert rc == a3d.A3D_E_UNSUPPORTED


def test_batch_rejects_bad_windows_without_gpu(engine_lib):
    """a3d_run_batch checks every window and shot before it touches a device."""
    import a3d
    import numpy as np
    cfg = a3d.make_config("iso", 12, 10, 8, nt=10)
    m = {"vel": np.full((10, 12, 8), 2000, np.float32), "rho": np.full((10, 12, 8), 2000, np.float32)}
    with pytest.raises(a3d.A3DError) as ei:
        a3d.run_batch(cfg, m, [(2, 2, 2)], windows=[(6, 0, 0, 8, 10, 8)])  # x0 + nx > 12
    assert ei.value.code == a3d.A3D_E_ARG and "outside the 12x10x8 model" in str(ei.value)
    with pytest.raises(a3d.A3DError) as ei:
        a3d.run_batch(cfg, m, [(1, 2, 2)], windows=[(2, 0, 0, 8, 10, 8)])  # shot left of its window
    assert ei.value.code == a3d.A3D_E_ARG and "outside its window" in str(ei.value)


def test_multishot_sweeps_only_for_vti(engine_lib):
    """cfg.batch > 1 (multi-shot sweeps) is built for the VTI engine with FP32 or
    2-byte storage; other physics and the FP64 run refuse it before any GPU work."""
    import a3d
    for phys, st in (("iso", a3d.FP32), ("tti", a3d.FP32), ("tti", a3d.FP16V), ("2o", a3d.FP32), ("vti", a3d.FP64)):
        cfg = a3d.make_config(phys, 10, 10, 10, storage=st, batch=4)
        h = ctypes.c_void_p()
        rc = a3d.lib().a3d_engine_create(ctypes.byref(h), ctypes.byref(cfg), *[a3d._fptr(None)] * 6, 0)
        assert rc == a3d.A3D_E_UNSUPPORTED, (phys, st, rc)
        assert "multi-shot" in a3d.last_error()
