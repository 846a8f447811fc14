"""Every launch configuration the autotuner can pick gives the same record.

The autotuner chooses, per kernel kind and grid, a tile width, rows per lane, ring
depth, sweep plan and (1st-order engines) the z-tile order; the parity tests see
only the configuration it picks on
their grids.  Here each configuration is pinned (A3D_TUNE) in turn and its record
compared bit for bit with the CPU oracle's engine form, on a grid with partial
tiles in z and x, a y split into several chunks, and PML on every face.
"""
import os

import numpy as np
import pytest

import oracle as O
from helpers import make_models

pytestmark = pytest.mark.gpu

SHAPES = {  # (tile width, rows per lane) built per physics
    "2o": [(8, 1), (16, 1), (8, 2), (16, 2), (16, 4)],
    "iso": [(8, 1), (16, 1), (8, 2), (16, 2), (16, 4)],          # the two-sweep step (A3D_FUSED=0)
    "iso_fused": [(8, 1), (16, 1), (8, 2), (16, 2)],             # the fused step, ring depths 0 and 1
    "vti": [(8, 1), (16, 1), (8, 2), (16, 2)],
    "tti": [(8, 1), (16, 1)],
}
CASE = {"2o": (30, 27, 45, (13, 11, 6), 70, 10), "iso": (30, 27, 45, (13, 11, 6), 70, 8),
        "iso_fused": (30, 27, 45, (13, 11, 6), 70, 8),
        "vti": (30, 27, 45, (13, 11, 6), 70, 8), "tti": (26, 23, 37, (11, 9, 5), 60, 8)}


def _configs(eng):
    out = []
    for tx, rows in SHAPES[eng]:
        for depth in ((0, 1) if eng == "iso_fused" else (0, 1, 2)):
            for plan in (0, 1, 2):
                out.append(f"{tx},{rows},{depth},{plan}")
                if eng != "2o":  # the same shape with the rotated z-tile order
                    out.append(f"{tx},{rows},{depth},{plan},1")
    return out


@pytest.fixture(autouse=True)
def _clear_tune():
    old = os.environ.pop("A3D_TUNE", None)
    oldf = os.environ.pop("A3D_FUSED", None)
    yield
    os.environ.pop("A3D_TUNE", None)
    os.environ.pop("A3D_FUSED", None)
    if old is not None:
        os.environ["A3D_TUNE"] = old
    if oldf is not None:
        os.environ["A3D_FUSED"] = oldf


@pytest.mark.parametrize("eng", ["2o", "iso", "iso_fused", "vti", "tti"])
def test_every_launch_configuration_matches_the_oracle(engine_lib, eng):
    import a3d
    nx, ny, nz, shot, nt, npml = CASE[eng]
    phys = "iso" if eng == "iso_fused" else eng
    if eng in ("iso", "iso_fused"):
        os.environ["A3D_FUSED"] = "1" if eng == "iso_fused" else "0"
    models = make_models(phys, nx, ny, nz, seed=21)
    s = O.Shot(nx, ny, nz, sx=shot[0], sy=shot[1], sz=shot[2], nt=nt, dt=1e-3, fm=25.0, npml=npml, rec_z=1,
               mute=False, form=1)
    ref, _ = O.run(phys, s, models, "f32")
    cfg = a3d.make_config(phys, nx, ny, nz, nt=nt, dt=1e-3, fm=25.0, npml=npml, rec_z=1)
    bad, ran, unfit = [], 0, []
    for c in _configs(eng):
        os.environ["A3D_TUNE"] = c if eng in ("2o", "iso_fused") else f"{c};{c}"
        e = a3d.Engine(cfg, models)
        try:
            rec = e.run(*shot)
        except a3d.A3DError as err:  # rings larger than a CTA's shared memory
            assert "invalid configuration" in str(err), str(err)
            unfit.append(c)
            continue
        finally:
            e.close()
        ran += 1
        if not np.array_equal(rec, ref):
            bad.append((c, int(np.count_nonzero(rec != ref))))
    assert not bad, f"configurations differing from the oracle: {bad}"
    assert ran >= len(unfit), f"too few configurations fit: {unfit}"
