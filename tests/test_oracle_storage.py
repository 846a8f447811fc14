"""The oracle's emulation of the engines' reduced-precision storage (CPU; test
infrastructure).

The engines store wavefields as bfloat16, as float16 of 2^k x (k the engine's
power-of-two scales), or (FP16V) u, v, w as scaled float16 with P, Q float; since
the scales are powers of two, the engine's arithmetic is the FP32 engine form times
powers of two, rounded where the engine stores.  The float oracle emulates that
with `store` = 1, 2, 4.  Here: the roundings against IEEE binary16 (numpy's
conversion: ties to even, subnormals, overflow) and known bfloat16 values, and the
emulated records against the double oracle.  tests/test_gpu_halfstore.py compares
the CUDA records with this emulation bit for bit.
"""
import numpy as np
import pytest

from helpers import make_models, rel_l2


def _round(xs):
    import oracle as O
    L = O.lib()
    return np.array([L.a3d_oracle_round_f16(float(x)) for x in xs], np.float32)


def test_round_f16_matches_ieee_binary16():
    rng = np.random.default_rng(3)
    mant = rng.uniform(1.0, 2.0, 4000).astype(np.float32)
    expo = rng.integers(-30, 17, 4000)
    xs = (mant * np.exp2(expo.astype(np.float32))).astype(np.float32)
    xs[::2] *= -1
    one = np.float32(1.0)
    ties = np.array([1 + 2.0 ** -11, 1 + 3 * 2.0 ** -11, 2048 + 1, 2048 + 3, 2.0 ** -25, 3 * 2.0 ** -25,
                     2.0 ** -14 + 2.0 ** -25, 65504.0, 65519.0, 65520.0, 70000.0, 0.0, -0.0, 6e-8, 5.96e-8,
                     2.0 ** -24, one], np.float32)
    xs = np.concatenate([xs, ties, -ties])
    with np.errstate(over="ignore"):
        want = xs.astype(np.float16).astype(np.float32)
    got = _round(xs)
    bad = ~((got == want) | (np.isinf(got) & np.isinf(want) & (np.sign(got) == np.sign(want))))
    assert not bad.any(), f"{int(bad.sum())} values differ, first {xs[bad][:4]} -> {got[bad][:4]} vs {want[bad][:4]}"


@pytest.mark.parametrize("physics", ["vti", "tti"])
def test_fp16v_emulation_error_vs_double_oracle(physics):
    """The emulated FP16V record differs from the float engine form and lies within
    the precision gate (1e-3) of the double oracle on a small case."""
    import oracle as O
    nx, ny, nz, nt = 24, 22, 20, 150
    m = make_models(physics, nx, ny, nz, seed=9)
    kw = dict(sx=11, sy=10, sz=4, nt=nt, dt=1e-3, fm=25.0, npml=8, form=1)
    r64, _ = O.run(physics, O.Shot(nx, ny, nz, **kw), m, "f64")
    r32, _ = O.run(physics, O.Shot(nx, ny, nz, **kw), m, "f32")
    k = 31 if physics == "vti" else 20  # the engine's velocity scales of such models (2^k * dx rho / dt range)
    r16, _ = O.run(physics, O.Shot(nx, ny, nz, store=4, sig_v_log2=k, **kw), m, "f32")
    assert not np.array_equal(r16, r32)
    err16, err32 = rel_l2(r16, r64), rel_l2(r32, r64)
    assert err32 < 2e-6 and err16 <= 1e-3 and err16 > 10 * err32, (err16, err32)


def test_round_bf16_known_values():
    import oracle as O
    L = O.lib()
    cases = [(1.0 + 2.0 ** -8, 1.0), (1.0 + 3 * 2.0 ** -8, 1.0 + 2.0 ** -6), (1.0 + 2.0 ** -9, 1.0),
             (-(1.0 + 2.0 ** -7 + 2.0 ** -9), -(1.0 + 2.0 ** -7)), (3.0e38, 3.0040553e38), (0.0, 0.0), (2.5, 2.5)]
    for x, want in cases:
        got = L.a3d_oracle_round_bf16(float(np.float32(x)))
        assert abs(got - want) <= abs(want) * 1e-4, (x, got, want)
    assert np.isinf(L.a3d_oracle_round_bf16(float(np.finfo(np.float32).max)))


@pytest.mark.parametrize("physics", ["iso", "vti", "tti"])
def test_two_byte_emulation_errors_order(physics):
    """Emulated bfloat16 and float16 storage: both differ from the float engine form;
    float16 (11-bit significand) lies closer to the double oracle than bfloat16 (8)."""
    import oracle as O
    nx, ny, nz, nt = 24, 22, 20, 150
    m = make_models(physics, nx, ny, nz, seed=9)
    kw = dict(sx=11, sy=10, sz=4, nt=nt, dt=1e-3, fm=25.0, npml=8, form=1)
    r64, _ = O.run(physics, O.Shot(nx, ny, nz, **kw), m, "f64")
    r32, _ = O.run(physics, O.Shot(nx, ny, nz, **kw), m, "f32")
    kv = 20 if physics == "tti" else (21 if physics == "iso" else 31)
    kp = -3 if physics == "iso" else 7
    err = {}
    for st in (1, 2):
        r, _ = O.run(physics, O.Shot(nx, ny, nz, store=st, sig_v_log2=kv, sig_p_log2=kp, **kw), m, "f32")
        assert not np.array_equal(r, r32)
        err[st] = rel_l2(r, r64)
    assert rel_l2(r32, r64) < err[2] < err[1] < 0.2, err



def test_round_f24_known_values():
    import oracle as O
    L = O.lib()
    one = np.float32(1.0)
    cases = [(1.0 + 2.0 ** -16, 1.0), (1.0 + 3 * 2.0 ** -16, 1.0 + 2.0 ** -14), (1.0 + 2.0 ** -15, 1.0 + 2.0 ** -15),
             (-(2.0 + 2.0 ** -15), -2.0), (0.0, 0.0), (float(one), 1.0)]
    for x, want in cases:
        got = L.a3d_oracle_round_f24(float(np.float32(x)))
        assert got == np.float32(want), (x, got, want)
    assert np.isinf(L.a3d_oracle_round_f24(float(np.finfo(np.float32).max)))


def test_f24_emulation_error_vs_double_oracle():
    """The 24-bit formats (no engine stores them yet): velocities only (store 6) and
    every field (store 5) lie far inside the precision gate on a small VTI case, and
    below the float16 forms' errors."""
    import oracle as O
    nx, ny, nz, nt = 24, 22, 20, 150
    m = make_models("vti", nx, ny, nz, seed=9)
    kw = dict(sx=11, sy=10, sz=4, nt=nt, dt=1e-3, fm=25.0, npml=8, form=1)
    r64, _ = O.run("vti", O.Shot(nx, ny, nz, **kw), m, "f64")
    err = {}
    for st in (2, 4, 5, 6):
        r, _ = O.run("vti", O.Shot(nx, ny, nz, store=st, sig_v_log2=31, sig_p_log2=7, **kw), m, "f32")
        err[st] = rel_l2(r, r64)
    assert err[6] < err[5] < 1e-3 and err[6] < err[4] and err[5] < err[2], err
