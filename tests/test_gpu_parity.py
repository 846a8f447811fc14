"""GPU parity: the CUDA engines against the CPU oracle, through the C ABI.

The engines perform exactly the oracle's engine-form operations (explicit fused
multiply-adds, no compiler contraction on either side), so for the FP32 path the
records must agree bit for bit.  The only exception is TTI's trig, where both
sides use host cosf/sinf; it is bitwise too.  The FP64 path (the FP64 oracle run
on the GPU) is checked against the double oracle at 1e-12.
"""
import numpy as np
import pytest

import oracle as O
from helpers import NPML_REF, make_models, rel_l2

pytestmark = pytest.mark.gpu

CASES = [
    # engine, nx, ny, nz, shot, nt, npml (None = reference), mute, wtype
    ("2o", 20, 18, 22, (9, 8, 5), 120, None, False, 1),
    ("2o", 33, 17, 40, (3, 15, 30), 90, 12, False, 1),
    ("2o", 16, 16, 16, (8, 8, 2), 200, 20, True, 1),
    ("iso", 20, 18, 16, (9, 8, 4), 220, None, True, 1),
    ("iso", 37, 21, 45, (1, 19, 43), 120, 8, False, 3),
    ("iso", 12, 12, 12, (5, 6, 3), 100, None, False, 6),
    ("vti", 20, 18, 16, (9, 8, 4), 220, None, True, 1),
    ("vti", 37, 21, 45, (30, 2, 10), 120, 8, False, 1),
    ("tti", 20, 18, 16, (9, 8, 4), 220, 12, True, 1),
    ("tti", 26, 19, 33, (4, 10, 6), 100, None, False, 1),
]


def _run_pair(a3d, eng, nx, ny, nz, shot, nt, npml, mute, wtype, storage, form_prec):
    models = make_models(eng, nx, ny, nz, seed=nx * 1000 + ny * 10 + nz)
    np_ = npml if npml else NPML_REF[eng]
    cfg = a3d.make_config(eng, nx, ny, nz, nt=nt, dt=1e-3, fm=25.0, wtype=wtype, npml=np_, rec_z=1,
                          mute=mute, storage=storage)
    e = a3d.Engine(cfg, models)
    try:
        rec = e.run(*shot)
    finally:
        e.close()
    s = O.Shot(nx, ny, nz, sx=shot[0], sy=shot[1], sz=shot[2], nt=nt, dt=1e-3, fm=25.0, wtype=wtype,
               npml=np_, rec_z=1, mute=mute, form=1)
    ref, _ = O.run(eng, s, models, form_prec)
    return rec, ref


@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]}-{c[1]}x{c[2]}x{c[3]}" for c in CASES])
def test_fp32_bitwise_vs_oracle(engine_lib, case):
    import a3d
    rec, ref = _run_pair(a3d, *case, storage=a3d.FP32, form_prec="f32")
    assert np.isfinite(rec).all()
    assert np.abs(ref).max() > 0
    mism = np.count_nonzero(rec != ref)
    assert mism == 0, f"{mism} of {rec.size} samples differ; rel-L2 {rel_l2(rec, ref):.3e}"


@pytest.mark.parametrize("case", CASES[::2], ids=[f"{c[0]}-{c[1]}x{c[2]}x{c[3]}" for c in CASES[::2]])
def test_fp64_vs_double_oracle(engine_lib, case):
    import a3d
    rec, ref = _run_pair(a3d, *case, storage=a3d.FP64, form_prec="f64")
    # the GPU record is stored as float; the double oracle is compared after rounding
    assert rel_l2(rec, ref.astype(np.float32)) < 1e-6


def test_snapshots_match_oracle(engine_lib):
    import a3d
    nx, ny, nz, nt = 20, 18, 16, 60
    models = make_models("iso", nx, ny, nz, seed=5)
    cfg = a3d.make_config("iso", nx, ny, nz, nt=nt, dt=1e-3, fm=25.0)
    e = a3d.Engine(cfg, models)
    rec, snaps = e.run(9, 8, 4, snap_every=20)
    e.close()
    s = O.Shot(nx, ny, nz, sx=9, sy=8, sz=4, nt=nt, dt=1e-3, fm=25.0, npml=20, form=1, snap_every=20)
    ref, rsn = O.run("iso", s, models, "f32", snaps=True)
    assert snaps.shape == rsn.shape
    assert np.array_equal(snaps, rsn)
    assert np.array_equal(rec, ref)


def test_shots_are_independent(engine_lib):
    """Running shot B after shot A gives the same record as running B alone."""
    import a3d
    nx, ny, nz, nt = 24, 20, 18, 80
    models = make_models("vti", nx, ny, nz, seed=9)
    cfg = a3d.make_config("vti", nx, ny, nz, nt=nt, dt=1e-3, fm=25.0, mute=True)
    e = a3d.Engine(cfg, models)
    e.run(3, 4, 2)
    b1 = e.run(20, 15, 6)
    e.close()
    e2 = a3d.Engine(cfg, models)
    b2 = e2.run(20, 15, 6)
    e2.close()
    assert np.array_equal(b1, b2)
