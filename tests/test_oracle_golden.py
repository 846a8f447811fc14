"""The CPU oracle against the reference's own CUDA kernels (golden records).

The golden records were produced by running the reference's kernels, built from
its sources, on a GB300 (tests/golden/make_golden.py).  Tolerance: the shot-record
relative L2 gate of the FP32 path, 1e-5, on the unmuted record; the mute is checked
sample by sample.  Both arithmetic forms of the oracle are pinned.
"""
import numpy as np
import pytest

import oracle as O
from golden_cases import NPML_REF, golden_files, load, mute_consistent
from helpers import rel_l2

FILES = golden_files()


def _shot(case, mute, form):
    return O.Shot(case["nx"], case["ny"], case["nz"], dx=case["dx"], dy=case["dy"], dz=case["dz"],
                  sx=case["sx"], sy=case["sy"], sz=case["sz"], nt=case["nt"], dt=case["dt"], fm=case["fm"],
                  wtype=case.get("wtype", 1), npml=NPML_REF[case["engine"]], rec_z=1, mute=mute, form=form)


def test_golden_files_present():
    names = {f.split("/")[-1] for f in FILES}
    for need in ("2o_a.npz", "iso_a.npz", "vti_a.npz", "tti_a.npz"):
        assert need in names


@pytest.mark.parametrize("path", FILES, ids=[f.split("/")[-1][:-4] for f in FILES])
@pytest.mark.parametrize("form", [0, 1])
def test_oracle_matches_reference(path, form):
    case, models, g = load(path)
    rec, _ = O.run(case["engine"], _shot(case, False, form), models, "f32")
    err = rel_l2(rec, g["rec"])
    assert err < 1e-5, f"rel-L2 {err:.3e}"
    if "rec_mute" in g:
        recm, _ = O.run(case["engine"], _shot(case, True, form), models, "f32")
        assert mute_consistent(g["rec"], g["rec_mute"], recm, rec)


def test_planted_error_is_caught():
    """A perturbed oracle (one model cell changed) fails the same gate."""
    case, models, g = load([f for f in FILES if f.endswith("iso_a.npz")][0])
    bad = dict(models)
    vel = bad["vel"].copy()
    vel[case["ny"] // 2, case["nx"] // 2, case["nz"] // 2] *= 1.01
    bad["vel"] = vel
    rec, _ = O.run("iso", _shot(case, False, 0), bad, "f32")
    assert rel_l2(rec, g["rec"]) > 1e-5
