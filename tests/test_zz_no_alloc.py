"""The 2nd-order step that allocates nothing (a3d_2order_step_noalloc).

It exists for callers that cannot call cudaMalloc (their device memory comes from
a pool they own, or is provisioned up front): they pass every buffer, and the
step's own scratch lives in a fixed array inside the library.  This test drives
whole shots through it, one call per time step, on buffers allocated by the test
(torch), and checks the records against the engine entry point (a3d_engine_run)
bit for bit — the tolerance of the FP32 parity tests — for two shots in a row, so
the second shot runs on scratch the first one left behind.  It also checks that a
grid beyond the stated limit is rejected before any GPU work.

The file name sorts last so that a run stopping at the first failure has already
run every other test.
"""
import ctypes
from ctypes import c_float, c_int, c_void_p

import numpy as np
import pytest

import oracle as O
from helpers import make_models

pytestmark = pytest.mark.gpu


def _step_fn(lib):
    fn = lib.a3d_2order_step_noalloc
    fn.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p] + [c_int] * 5 + [c_float] * 3 + \
                  [c_int] * 3 + [c_float] + [c_int] * 4
    fn.restype = c_int
    return fn


def _noalloc_shot(step, torch, vel, nx, ny, nz, npd, shot, nt, dt, fm, rec_z):
    pad = 4 + npd
    nnx, nny, nnz = nx + 2 * pad, ny + 2 * pad, nz + 2 * pad
    ldz = (nnz + 3) // 4 * 4
    # (v dt)^2, edge-padded, rows of ldz floats
    vp = np.pad(vel, pad, mode="edge").astype(np.float32)
    t = vp * np.float32(dt)
    vv_img = np.zeros((nny, nnx, ldz), np.float32)
    vv_img[:, :, :nnz] = t * t
    dev = torch.device("cuda:0")
    vv = torch.from_numpy(vv_img).to(dev)
    buf = [torch.zeros((nny, nnx, ldz), dtype=torch.float32, device=dev) for _ in range(2)]
    rec = torch.zeros((ny, nx, nt), dtype=torch.float32, device=dev)
    w = [O.lib().a3d_oracle_ricker2o(it, dt, fm) for it in range(nt)]
    sx, sy, sz = shot
    buf[0][sy + pad, sx + pad, sz + pad] = w[0]
    buf[0][sy + pad, sx + pad, sz + pad + 2] = -w[0]
    torch.cuda.synchronize()
    cur = 0
    for it in range(nt):
        rc = step(buf[cur].data_ptr(), buf[1 - cur].data_ptr(), vv.data_ptr(), rec.data_ptr(),
                  nx, ny, nz, npd, ldz, 10.0, 10.0, 10.0, sx, sy, sz,
                  w[it + 1] if it + 1 < nt else 0.0, rec_z, it, nt, 0)
        assert rc == 0, f"step {it} returned {rc}"
        cur = 1 - cur
    return rec.cpu().numpy()


def test_noalloc_step_matches_engine_two_shots(engine_lib):
    torch = pytest.importorskip("torch")
    import a3d
    step = _step_fn(a3d.lib())
    nx, ny, nz, npd, nt, dt, fm = 20, 18, 22, 20, 80, 1e-3, 25.0
    models = make_models("2o", nx, ny, nz, seed=77)
    cfg = a3d.make_config("2o", nx, ny, nz, nt=nt, dt=dt, fm=fm, npml=npd, rec_z=1)
    e = a3d.Engine(cfg, models)
    try:
        for shot in ((9, 8, 5), (3, 14, 9)):  # two shots in a row through the same scratch
            ref = e.run(*shot)
            got = _noalloc_shot(step, torch, models["vel"], nx, ny, nz, npd, shot, nt, dt, fm, 1)
            assert np.abs(ref).max() > 0
            assert np.array_equal(got, ref), f"shot {shot}: {np.count_nonzero(got != ref)} samples differ"
    finally:
        e.close()


def test_noalloc_step_rejects_oversize_grid(engine_lib):
    import a3d
    step = _step_fn(a3d.lib())
    big = 4200  # padded axis 4200 + 8 + 40 > the 4096-cell limit
    rc = step(16, 16, 16, None, big, 8, 8, 20, 64, 10.0, 10.0, 10.0, 1, 1, 1, 0.0, 1, 0, 10, 0)
    assert rc == a3d.A3D_E_ARG
    assert "limit" in a3d.last_error()
    # every axis within the limit (1400 + 8 + 40 = 1448 cells), but 1448^3 cells
    # exceed the 2^31 - 1 cells the step's 32-bit offsets reach; rejected before any
    # GPU work, so the fake pointers are never touched
    n, npd = 1400, 20
    rc = step(16, 16, 16, None, n, n, n, npd, 1448, 10.0, 10.0, 10.0, 1, 1, 1, 0.0, 1, 0, 10, 0)
    assert rc == a3d.A3D_E_ARG
    assert "2^31" in a3d.last_error()
