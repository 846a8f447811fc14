"""GPU checks of the batched multi-shot entry point (a3d_run_batch).

A batch must give, shot for shot, the records of single-shot engine runs: the
whole-model shots those of one engine on the model, the windowed shots those of
an engine (and of the CPU oracle) on the model cropped to the window, and the
CUDA-graph replay of the time loop those of the plain stream launches.
"""
import numpy as np
import pytest

import oracle as O
from helpers import NPML_REF, make_models

pytestmark = pytest.mark.gpu


def _cfg(a3d, eng, nx, ny, nz, nt, npml=None, mute=False):
    return a3d.make_config(eng, nx, ny, nz, nt=nt, dt=1e-3, fm=25.0, npml=npml or NPML_REF[eng], rec_z=1,
                           mute=mute)


@pytest.mark.parametrize("eng", ["2o", "iso", "vti"])
def test_whole_model_batch_equals_single_runs(engine_lib, eng):
    import a3d
    nx, ny, nz, nt = 22, 18, 20, 90
    models = make_models(eng, nx, ny, nz, seed=7)
    cfg = _cfg(a3d, eng, nx, ny, nz, nt, npml=10 if eng != "2o" else 12, mute=True)
    shots = [(5, 6, 3), (16, 9, 4), (11, 11, 2)]
    recs, ms = a3d.run_batch(cfg, models, shots)
    e = a3d.Engine(cfg, models)
    try:
        for i, s in enumerate(shots):
            ref = e.run(*s)
            assert np.array_equal(recs[i], ref), f"shot {i} differs"
            assert ms[i] > 0
    finally:
        e.close()


@pytest.mark.parametrize("eng", ["iso", "tti"])
def test_windowed_batch_equals_cropped_model(engine_lib, eng):
    import a3d
    nx, ny, nz, nt = 40, 34, 30, 80
    models = make_models(eng, nx, ny, nz, seed=11)
    npml = 8
    cfg = _cfg(a3d, eng, nx, ny, nz, nt, npml=npml)
    windows = [(3, 2, 0, 24, 20, 22), (10, 9, 5, 26, 22, 20), (10, 9, 5, 26, 22, 20), (0, 0, 0, 0, 0, 0)]
    shots = [(3 + 12, 2 + 10, 2), (10 + 13, 9 + 11, 7), (10 + 5, 9 + 4, 9), (20, 17, 2)]
    recs, _ = a3d.run_batch(cfg, models, shots, windows=windows)
    for i, (w, s) in enumerate(zip(windows, shots)):
        if w[3] == 0:
            assert recs[i].shape == (ny, nx, nt)
            continue
        x0, y0, z0, wx, wy, wz = w
        crop = {k: v.reshape(ny, nx, nz)[y0:y0 + wy, x0:x0 + wx, z0:z0 + wz].copy() for k, v in models.items()}
        rel = (s[0] - x0, s[1] - y0, s[2] - z0)
        sh = O.Shot(wx, wy, wz, sx=rel[0], sy=rel[1], sz=rel[2], nt=nt, dt=1e-3, fm=25.0, npml=npml, rec_z=1,
                    mute=False, form=1)
        ref, _ = O.run(eng, sh, crop, "f32")
        assert recs[i].shape == (wy, wx, nt)
        assert np.array_equal(recs[i], ref), f"windowed shot {i} differs from the oracle on its window"


@pytest.mark.parametrize("eng", ["2o", "iso", "tti"])
def test_graph_replay_equals_stream_launches(engine_lib, eng):
    import a3d
    nx, ny, nz, nt = 20, 18, 16, 70
    models = make_models(eng, nx, ny, nz, seed=3)
    cfg = _cfg(a3d, eng, nx, ny, nz, nt, npml=10 if eng != "2o" else 12)
    shots = [(9, 8, 4), (4, 12, 3)]
    plain, _ = a3d.run_batch(cfg, models, shots, graph=False)
    graph, ms = a3d.run_batch(cfg, models, shots, graph=True)
    for a, b in zip(plain, graph):
        assert np.abs(a).max() > 0
        assert np.array_equal(a, b)
    assert all(m > 0 for m in ms)
