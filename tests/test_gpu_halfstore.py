"""GPU checks of reduced-precision wavefield storage (isotropic, VTI and TTI engines).

The wavefields u, v, w, P and the split PML components are stored as bfloat16 or
float16 (float16 with power-of-two per-field scales); every stencil operation and
the time integration stay float.  FP16V (VTI, TTI) stores u, v, w as float16 and
P, Q and their split components as float.  Each form's record is compared bit for
bit with the float oracle's emulation of its storage
(test_reduced_storage_bitwise_vs_oracle_emulation), and its error with the same
shot run in FP64 storage.

FP16V is held to the 1e-3 precision gate, on the 300-step case and on a 1500-step
record of the same model (measured on GB300: VTI 9.0e-4 and 9.3e-4, TTI 9.2e-4 and
9.6e-4).  The all-2-byte
forms do not meet that gate; their bounds are regression guards at about 2x the
stated error of each form on this case (measured on GB300: bfloat16 4.7e-2,
float16 4.4e-3, FP32 7.7e-7), not the precision target.
"""
import numpy as np
import pytest

from helpers import make_models, rel_l2

pytestmark = pytest.mark.gpu

NX, NY, NZ, NT = 40, 36, 32, 300
SHOT = (18, 17, 4)
TOL = {"bf16": 1e-1, "fp16": 1e-2, "fp32": 2e-6}


def _run(a3d, storage, models, mute=False):
    cfg = a3d.make_config("iso", NX, NY, NZ, nt=NT, dt=1e-3, fm=25.0, npml=10, storage=storage, mute=mute)
    e = a3d.Engine(cfg, models)
    try:
        return e.run(*SHOT)
    finally:
        e.close()


@pytest.fixture(scope="module")
def fp64_record(engine_lib):
    import a3d
    models = make_models("iso", NX, NY, NZ, seed=5)
    return models, _run(a3d, a3d.FP64, models)


@pytest.mark.parametrize("name", ["bf16", "fp16", "fp32"])
def test_record_error_vs_fp64_within_stated_bound(engine_lib, fp64_record, name):
    import a3d
    models, ref = fp64_record
    code = {"bf16": a3d.BF16, "fp16": a3d.FP16, "fp32": a3d.FP32}[name]
    rec = _run(a3d, code, models)
    assert np.isfinite(rec).all()
    assert np.abs(rec).max() > 0
    err = rel_l2(rec, ref)
    assert err <= TOL[name], f"{name}: rel-L2 vs FP64 {err:.3e} above {TOL[name]:.0e}"


def test_half_storage_mutes_the_same_samples(engine_lib, fp64_record):
    """Samples the direct-wave mute zeroes in FP32 are zero with float16 storage too."""
    import a3d
    models, _ = fp64_record
    muted = (_run(a3d, a3d.FP32, models, mute=True) == 0) & (_run(a3d, a3d.FP32, models) != 0)
    assert muted.any()
    r16 = _run(a3d, a3d.FP16, models, mute=True)
    assert np.all(r16[muted] == 0)


PRECISION_GATE = 1e-3


@pytest.mark.parametrize("name,tol,nt", [("bf16", 5e-2, NT), ("fp16", 5e-3, NT), ("fp32", 2e-6, NT),
                                         ("fp16v", PRECISION_GATE, NT), ("fp16v", PRECISION_GATE, 1500)],
                         ids=["bf16", "fp16", "fp32", "fp16v", "fp16v-1500"])
def test_vti_record_error_vs_fp64_within_stated_bound(engine_lib, name, tol, nt):
    """VTI with reduced-precision storage (measured on the 300-step case: bfloat16
    2.4e-2, float16 2.4e-3, FP32 6.7e-7, FP16V 9.0e-4; FP16V after 1500 steps
    9.3e-4, where bfloat16 has diverged)."""
    import a3d
    models = make_models("vti", NX, NY, NZ, seed=5)
    code = {"bf16": a3d.BF16, "fp16": a3d.FP16, "fp32": a3d.FP32, "fp16v": a3d.FP16V}[name]
    recs = {}
    for key, st in (("ref", a3d.FP64), ("run", code)):
        cfg = a3d.make_config("vti", NX, NY, NZ, nt=nt, dt=1e-3, fm=25.0, npml=10, storage=st)
        e = a3d.Engine(cfg, models)
        try:
            recs[key] = e.run(*SHOT)
        finally:
            e.close()
    assert np.isfinite(recs["run"]).all()
    err = rel_l2(recs["run"], recs["ref"])
    assert err <= tol, f"VTI {name}: rel-L2 vs FP64 {err:.3e} above {tol:.0e}"


@pytest.mark.parametrize("name,tol,nt", [("bf16", 5e-2, NT), ("fp16", 5e-3, NT), ("fp32", 2e-6, NT),
                                         ("fp16v", PRECISION_GATE, NT), ("fp16v", PRECISION_GATE, 1500)],
                         ids=["bf16", "fp16", "fp32", "fp16v", "fp16v-1500"])
def test_tti_record_error_vs_fp64_within_stated_bound(engine_lib, name, tol, nt):
    """TTI with reduced-precision storage (no density; tilt and azimuth varying
    gently, as the reference's update requires; measured on the 300-step case:
    bfloat16 2.2e-2, float16 2.6e-3, FP32 4.8e-7, FP16V 9.2e-4; FP16V after 1500
    steps 9.6e-4, where bfloat16 has diverged)."""
    import a3d
    models = make_models("tti", NX, NY, NZ, seed=5)
    code = {"bf16": a3d.BF16, "fp16": a3d.FP16, "fp32": a3d.FP32, "fp16v": a3d.FP16V}[name]
    recs = {}
    for key, st in (("ref", a3d.FP64), ("run", code)):
        cfg = a3d.make_config("tti", NX, NY, NZ, nt=nt, dt=1e-3, fm=25.0, npml=10, storage=st)
        e = a3d.Engine(cfg, models)
        try:
            recs[key] = e.run(*SHOT)
        finally:
            e.close()
    assert np.isfinite(recs["run"]).all()
    assert np.abs(recs["ref"]).max() > 0
    err = rel_l2(recs["run"], recs["ref"])
    print(f"TTI {name}: rel-L2 vs FP64 {err:.3e}")
    assert err <= tol, f"TTI {name}: rel-L2 vs FP64 {err:.3e} above {tol:.0e}"


def test_tti_fp16v_every_launch_shape(engine_lib):
    """TTI FP16V: every tile width and ring depth built for it gives the record of
    the tuned launch, bit for bit."""
    import os
    import a3d
    models = make_models("tti", 30, 27, 45, seed=41)

    def run(tune):
        old = os.environ.pop("A3D_TUNE", None)
        if tune:
            os.environ["A3D_TUNE"] = tune
        try:
            cfg = a3d.make_config("tti", 30, 27, 45, nt=120, dt=1e-3, fm=25.0, npml=8, storage=a3d.FP16V)
            e = a3d.Engine(cfg, models)
            try:
                return e.run(13, 11, 6)
            finally:
                e.close()
        finally:
            os.environ.pop("A3D_TUNE", None)
            if old is not None:
                os.environ["A3D_TUNE"] = old

    ref = run(None)
    assert np.isfinite(ref).all() and np.abs(ref).max() > 0
    for tx in (8, 16):
        for depth in (0, 2):
            r = run(f"{tx},1,{depth},0")
            assert np.array_equal(r, ref), f"{tx},1,{depth}: {np.count_nonzero(r != ref)} samples differ"


@pytest.mark.parametrize("physics", ["vti", "tti"])
def test_fp16v_snapshots_follow_the_fp32_run(engine_lib, physics):
    """FP16V snapshots crop the float P field.  A volume snapshot carries the
    rounding error accumulated up to its step over the whole field, which grows in
    time (VTI, measured: below 1e-3 at step 100, 7.4e-3 at step 200, where the
    record of the first 300 steps is 9.0e-4 off), so the bound here is 2e-2 against
    the FP32 snapshots, and every FP16V snapshot must be closer to them than the
    all-float16 run's; the record equals that of a run without snapshots."""
    import a3d
    models = make_models(physics, NX, NY, NZ, seed=5)
    out = {}
    for st in (a3d.FP32, a3d.FP16V, a3d.FP16):
        cfg = a3d.make_config(physics, NX, NY, NZ, nt=NT, dt=1e-3, fm=25.0, npml=10, storage=st)
        e = a3d.Engine(cfg, models)
        try:
            out[st] = e.run(*SHOT, snap_every=100, snap_skip0=True)
            if st == a3d.FP16V:
                plain = e.run(*SHOT)
        finally:
            e.close()
    snaps32 = out[a3d.FP32][1]
    rec16v, snaps16v = out[a3d.FP16V]
    snaps16 = out[a3d.FP16][1]
    assert snaps16v.shape == snaps32.shape == (2, NY, NX, NZ)
    assert np.array_equal(rec16v, plain)
    for k in range(snaps32.shape[0]):
        assert np.abs(snaps32[k]).max() > 0
        err = rel_l2(snaps16v[k], snaps32[k])
        err16 = rel_l2(snaps16[k], snaps32[k])
        print(f"{physics} snapshot {k}: FP16V {err:.3e}, float16 {err16:.3e}")
        assert err <= 2e-2 and err < err16, f"{physics} snapshot {k}: FP16V {err:.3e}, float16 {err16:.3e}"


EMU_CASES = [("vti", "fp16v", False), ("tti", "fp16v", False), ("vti", "fp16v", True), ("iso", "bf16", False),
             ("iso", "fp16", False), ("iso", "fp16", True), ("vti", "bf16", False), ("vti", "fp16", False),
             ("tti", "bf16", False), ("tti", "fp16", False)]


@pytest.mark.parametrize("physics,storage,mute", EMU_CASES,
                         ids=[f"{p}-{s}" + ("-mute" if m else "") for p, s, m in EMU_CASES])
def test_reduced_storage_bitwise_vs_oracle_emulation(engine_lib, physics, storage, mute):
    """Reduced-precision records equal, bit for bit, the float oracle's engine form
    with the engine's storage emulated (oracle `store`): every stored field rounded
    where the engine stores it — bfloat16, float16 of 2^k x with the engine's scales
    k, or (FP16V) float16 u, v, w with float P, Q — the velocity sweep's view of the
    injected source rounded as the engine rounds it, and the record sampled before
    the pressure is rounded; snapshots (the stored pressure) too.  The scales are
    powers of two, so scaled storage is the FP32 arithmetic times exact powers of
    two, rounded where the engine stores."""
    import a3d
    import oracle as O
    models = make_models(physics, NX, NY, NZ, seed=5)
    code = {"bf16": a3d.BF16, "fp16": a3d.FP16, "fp16v": a3d.FP16V}[storage]
    cfg = a3d.make_config(physics, NX, NY, NZ, nt=NT, dt=1e-3, fm=25.0, npml=10, storage=code, mute=mute)
    e = a3d.Engine(cfg, models)
    try:
        rec, snaps = e.run(*SHOT, snap_every=100, snap_skip0=True)
        d = e.describe()
    finally:
        e.close()
    s = O.Shot(NX, NY, NZ, sx=SHOT[0], sy=SHOT[1], sz=SHOT[2], nt=NT, dt=1e-3, fm=25.0, npml=10, mute=mute, form=1,
               snap_every=100, snap_skip0=True, store=code, sig_v_log2=d["sig_v_log2"], sig_p_log2=d["sig_p_log2"])
    ref, rsn = O.run(physics, s, models, "f32", snaps=True)
    assert np.abs(ref).max() > 0
    assert np.array_equal(rec, ref), f"{int(np.count_nonzero(rec != ref))} samples differ (scales {d['sig_v_log2']}, " \
                                     f"{d['sig_p_log2']})"
    assert snaps.shape == rsn.shape and np.array_equal(snaps, rsn), "snapshots differ"
