"""The batched survey driver (FD.survey: one process per GPU feeding a3d_run_batch)
writes the same shot files, byte for byte, as the legacy per-shot entry points
that readmodel.py calls, and resumes by skipping complete files."""
import os

import numpy as np
import pytest

from helpers import make_models

pytestmark = pytest.mark.gpu


def _setup(R, eng, tmp_path, sub):
    nx, ny, nz = 22, 18, 16
    models = make_models(eng, nx, ny, nz, seed=41)
    files = {}
    for k, a in models.items():
        files[k] = str(tmp_path / f"{k}.bin")
        a.tofile(files[k])
    m = R.Model(nx, ny, nz, 10.0, 10.0, 10.0, vel_file=files.get("vel"), rho_file=files.get("rho"),
                delta_file=files.get("del"), epsilon_file=files.get("eps"), theta_file=files.get("theta"),
                psi_file=files.get("phi"))
    out = tmp_path / sub
    out.mkdir()
    sg = R.ShotReceiver(sxbeg=6, sybeg=5, szbeg=3, jsx=8, jsy=7, jsz=1, sxend=14, syend=12, szend=3,
                        dgx=20.0, dgy=10.0, dgt=2e-3, shotfolder=str(out) + "/")
    cls = {"2o": R.Acoustic3d2order, "iso": R.Acoustic3d1order, "vti": R.Acoustic3dvti,
           "tti": R.Acoustic3dtti}[eng]
    return cls(m, sg, nt=100, dt=1e-3, fpeak=25.0, snap_folder=str(out) + "/", snap_interval=50,
               cut_directwave=eng != "2o")


@pytest.mark.parametrize("eng", ["2o", "iso", "vti", "tti"])
def test_survey_files_equal_legacy_files(engine_lib, tmp_path, eng):
    import readmodel as R
    legacy = _setup(R, eng, tmp_path, "legacy")
    for t in legacy.sg.nodetask[0]:
        legacy.run(t, 0)
    batched = _setup(R, eng, tmp_path, "batched")
    assert batched.survey(devices=(0,)) == batched.sg.nshot == 4
    for t in legacy.sg.nodetask[0]:
        a = open(legacy.shot_name(t), "rb").read()
        b = open(batched.shot_name(t), "rb").read()
        assert len(a) == legacy.record_bytes() and a == b, f"shot {t[:3]} differs"
    # resume: complete files are kept, nothing runs
    assert batched.survey(devices=(0,), skip_existing=True) == 0
    os.remove(batched.shot_name(batched.sg.nodetask[0][1]))
    assert batched.survey(devices=(0,), skip_existing=True) == 1
    t = batched.sg.nodetask[0][1]
    assert open(batched.shot_name(t), "rb").read() == open(legacy.shot_name(t), "rb").read()


@pytest.mark.parametrize("eng", ["vti", "tti"])
def test_fp16v_survey_writes_the_engine_records(engine_lib, tmp_path, eng):
    """storage="fp16v": each record file holds the FP16V engine's record of its shot
    in the legacy layout (VTI in multi-shot sweeps of 3, TTI one shot at a time)."""
    import a3d
    import readmodel as R
    fd = _setup(R, eng, tmp_path, "fp16v")
    assert fd.survey(devices=(0,), batch=3 if eng == "vti" else 0, storage="fp16v") == 4
    cfg = fd.engine_config()
    cfg.storage = a3d.FP16V
    e = a3d.Engine(cfg, fd.read_models())
    try:
        for t in fd.sg.nodetask[0]:
            rec = e.run(*t[:3])
            want = str(tmp_path / "want.bin")
            fd.write_record(want, rec)
            assert open(fd.shot_name(t), "rb").read() == open(want, "rb").read(), f"shot {t[:3]}"
    finally:
        e.close()


def test_vti_survey_in_multishot_sweeps(engine_lib, tmp_path):
    """batch=3 over the node's 4 shots: one sweep of 3 and one of 1, the record files
    of both written while the other runs, byte for byte the legacy entry point's."""
    import readmodel as R
    legacy = _setup(R, "vti", tmp_path, "legacy")
    for t in legacy.sg.nodetask[0]:
        legacy.run(t, 0)
    batched = _setup(R, "vti", tmp_path, "sweeps")
    assert batched.survey(devices=(0,), batch=3) == 4
    for t in legacy.sg.nodetask[0]:
        assert open(batched.shot_name(t), "rb").read() == open(legacy.shot_name(t), "rb").read()
