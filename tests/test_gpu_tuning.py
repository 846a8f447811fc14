"""The autotuner's choices: the isotropic step's two forms give the same record, and
an engine made again for the same grid reuses the tuned shapes (no second tuning)."""
import os
import time

import numpy as np
import pytest

from helpers import make_models

pytestmark = pytest.mark.gpu

NX, NY, NZ, NT = 40, 36, 44, 80
SHOT = (19, 17, 5)


@pytest.fixture(autouse=True)
def _clean_env():
    saved = {k: os.environ.pop(k, None) for k in ("A3D_TUNE", "A3D_FUSED")}
    yield
    for k, v in saved.items():
        os.environ.pop(k, None)
        if v is not None:
            os.environ[k] = v


def _record(a3d, models, **kw):
    cfg = a3d.make_config("iso", NX, NY, NZ, nt=NT, dt=1e-3, fm=25.0, npml=10, **kw)
    e = a3d.Engine(cfg, models)
    try:
        d = e.describe()
        return e.run(*SHOT), d
    finally:
        e.close()


def test_both_step_forms_give_the_same_record(engine_lib):
    import a3d
    models = make_models("iso", NX, NY, NZ, seed=31)
    os.environ["A3D_FUSED"] = "1"
    fused, d1 = _record(a3d, models)
    os.environ["A3D_FUSED"] = "0"
    two, d0 = _record(a3d, models)
    assert d1["fused"] == 1 and d0["fused"] == 0
    assert np.abs(two).max() > 0
    assert np.array_equal(fused, two)


def test_tuned_shapes_are_reused_for_the_same_grid(engine_lib):
    import a3d
    models = make_models("iso", NX, NY, NZ, seed=32)
    r1, d1 = _record(a3d, models, tile_x=0)
    t0 = time.perf_counter()
    r2, d2 = _record(a3d, models, tile_x=0)
    second = time.perf_counter() - t0
    assert d1["kernels"] == d2["kernels"] and d1["fused"] == d2["fused"]
    assert np.array_equal(r1, r2)
    # the second engine ran no candidate launches: its set-up and shot take well under
    # the tuner's dozens of timed launches on this grid
    assert second < 5.0
    # a pinned shape bypasses the cache and is taken as given, the z-tile order too
    os.environ["A3D_TUNE"] = "8,1,0,0;8,1,0,0,1"
    r3, d3 = _record(a3d, models, tile_x=0)
    assert d3["kernels"][0]["tile_x"] == 8 and d3["kernels"][0]["rows"] == 1 and d3["fused"] == 0
    assert d3["kernels"][0]["rot"] == 0 and d3["kernels"][1]["rot"] == 1
    assert np.array_equal(r3, r1)
