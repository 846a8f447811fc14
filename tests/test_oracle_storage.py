"""The oracle's emulation of the engines' FP16V storage (CPU; test infrastructure).

FP16V keeps u, v, w as float16 values of 2^k u (k the engine's velocity scale) and
P, Q as float; since the scales are powers of two, the engine's arithmetic is the
FP32 engine form times powers of two, rounded where the engine stores.  The float
oracle emulates that with `store = 4`: after every velocity update it rounds u, v,
w to the float16 grid of the scaled value.  Here: the rounding against numpy's IEEE
binary16 conversion (ties to even, subnormals, overflow), and the emulated records
against the double oracle.  tests/test_gpu_halfstore.py compares the CUDA FP16V
records with this emulation bit for bit.
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
