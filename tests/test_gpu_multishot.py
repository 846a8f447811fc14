"""Multi-shot sweeps of the VTI engine (cfg.batch = K, a3d_engine_run_shots).

One launch advances K shots of one model; each shot's arithmetic is that of a
one-shot run, so every record must equal the record of the same shot run alone
(a3d_engine_run on an engine without batching) bit for bit — FP32 and 2-byte
storage, mute on and off, a sweep over fewer shots than the engine holds, every
launch shape built for the multi-shot kernels, and through a3d_run_batch, which
groups consecutive shots on one window into sweeps.
"""
import os

import numpy as np
import pytest

from helpers import make_models

pytestmark = pytest.mark.gpu

NX, NY, NZ, NT, NPML = 30, 27, 45, 70, 8
NT_MUTE = 250  # the mute keeps no sample before arrival + 2 / (dt fm) + 60 = 140+ steps
SHOTS = [(13, 11, 6), (2, 25, 1), (28, 0, 40), (15, 14, 20)]


def _cfg(a3d, batch=0, storage=0, mute=False):
    return a3d.make_config("vti", NX, NY, NZ, nt=NT_MUTE if mute else NT, dt=1e-3, fm=25.0, npml=NPML,
                           storage=storage, mute=mute, batch=batch)


def _singles(a3d, models, shots, storage=0, mute=False):
    e = a3d.Engine(_cfg(a3d, storage=storage, mute=mute), models)
    try:
        return [e.run(*s) for s in shots]
    finally:
        e.close()


@pytest.fixture(scope="module")
def models():
    return make_models("vti", NX, NY, NZ, seed=41)


@pytest.fixture(autouse=True)
def _clear_tune():
    old = os.environ.pop("A3D_TUNE", None)
    yield
    os.environ.pop("A3D_TUNE", None)
    if old is not None:
        os.environ["A3D_TUNE"] = old


@pytest.mark.parametrize("storage,mute", [(0, False), (0, True), (2, False), (1, True), (4, False), (4, True)],
                         ids=["fp32", "fp32-mute", "fp16", "bf16-mute", "fp16v", "fp16v-mute"])
def test_sweep_records_equal_single_runs(engine_lib, models, storage, mute):
    import a3d
    ref = _singles(a3d, models, SHOTS, storage, mute)
    e = a3d.Engine(_cfg(a3d, batch=len(SHOTS), storage=storage, mute=mute), models)
    try:
        recs = e.run_shots(SHOTS)
        part = e.run_shots(SHOTS[1:])  # fewer shots than the engine holds, on fields the first sweep left
    finally:
        e.close()
    assert np.abs(ref[0]).max() > 0  # the shallow first shot keeps samples even when muted
    for j, r in enumerate(ref):
        assert np.array_equal(recs[j], r), f"shot {j}: {np.count_nonzero(recs[j] != r)} samples differ"
    for j, r in enumerate(ref[1:]):
        assert np.array_equal(part[j], r), f"partial sweep, shot {j + 1}"


def _ms_configs():
    out = []
    for tx, rows in ((8, 1), (16, 1), (8, 2), (16, 2)):
        for depth in (0, 2):
            for plan in (0, 1, 2):
                out.append(f"{tx},{rows},{depth},{plan}")
        out.append(f"{tx},{rows},0,0,1")  # rotated z-tile order
        for sblk in (3, 7, 10000):  # tile blocks (Sweep::sblk): partial last block, one past the grid
            out.append(f"{tx},{rows},0,2,0,{sblk}")
            out.append(f"{tx},{rows},2,0,1,{sblk}")
    return out


def test_every_multishot_launch_shape(engine_lib, models):
    import a3d
    ref = _singles(a3d, models, SHOTS[:3])
    for tune in _ms_configs():
        os.environ["A3D_TUNE"] = tune
        e = a3d.Engine(_cfg(a3d, batch=3), models)
        try:
            recs = e.run_shots(SHOTS[:3])
        finally:
            e.close()
        for j, r in enumerate(ref):
            assert np.array_equal(recs[j], r), f"A3D_TUNE={tune} shot {j}: {np.count_nonzero(recs[j] != r)} differ"


def test_every_fp16v_launch_shape(engine_lib, models):
    """float16 u, v, w with float P, Q (FP16V): every tile shape and ring depth built
    for it, one shot and multi-shot, gives the same records."""
    import a3d
    ref = _singles(a3d, models, SHOTS[:2], storage=a3d.FP16V)
    for tx, rows in ((8, 1), (16, 1), (16, 2)):
        for depth in (0, 2):
            os.environ["A3D_TUNE"] = f"{tx},{rows},{depth},0"
            one = _singles(a3d, models, SHOTS[:2], storage=a3d.FP16V)
            os.environ["A3D_TUNE"] = f"{tx},{rows},{depth},2,0,5"
            e = a3d.Engine(_cfg(a3d, batch=2, storage=a3d.FP16V), models)
            try:
                recs = e.run_shots(SHOTS[:2])
            finally:
                e.close()
            for j, r in enumerate(ref):
                assert np.array_equal(one[j], r), f"one shot, {tx},{rows},{depth}: shot {j}"
                assert np.array_equal(recs[j], r), f"sweep, {tx},{rows},{depth}: shot {j}"


@pytest.mark.parametrize("storage", [0, 4], ids=["fp32", "fp16v"])
def test_run_batch_groups_shots_into_sweeps(engine_lib, models, storage):
    import a3d
    shots = SHOTS + [(5, 5, 5)]
    ref = _singles(a3d, models, shots, storage)
    recs, ms = a3d.run_batch(_cfg(a3d, batch=3, storage=storage), models, shots, graph=True)
    assert len(recs) == len(shots) and all(t > 0 for t in ms)
    for j, r in enumerate(ref):
        assert np.array_equal(recs[j], r), f"shot {j}"


def test_single_shot_on_a_batch_engine(engine_lib, models):
    """run() on an engine of multi-shot sweeps is a sweep of one shot."""
    import a3d
    ref = _singles(a3d, models, SHOTS[:1])[0]
    e = a3d.Engine(_cfg(a3d, batch=2), models)
    try:
        rec = e.run(*SHOTS[0])
        one = e.record(0)
    finally:
        e.close()
    assert np.array_equal(rec, ref)
    assert np.array_equal(one, ref)
