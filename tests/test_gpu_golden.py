"""The CUDA engines against the reference's own CUDA kernels (golden records).

Gate: shot-record relative L2 <= 1e-5 for the FP32 path on the unmuted record
(the project's parity gate); the muted record must zero exactly the samples the
reference zeroed.
"""
import numpy as np
import pytest

from golden_cases import NPML_REF, golden_files, load, mute_consistent
from helpers import rel_l2

pytestmark = pytest.mark.gpu
FILES = golden_files()


@pytest.mark.parametrize("path", FILES, ids=[f.split("/")[-1][:-4] for f in FILES])
def test_engine_matches_reference(engine_lib, path):
    import a3d
    case, models, g = load(path)
    recs = {}
    for mute in (False, True):
        cfg = a3d.make_config(case["engine"], case["nx"], case["ny"], case["nz"], dx=case["dx"], dy=case["dy"],
                              dz=case["dz"], nt=case["nt"], dt=case["dt"], fm=case["fm"],
                              wtype=case.get("wtype", 1), npml=NPML_REF[case["engine"]], rec_z=1, mute=mute)
        e = a3d.Engine(cfg, models)
        recs[mute] = e.run(case["sx"], case["sy"], case["sz"])
        e.close()
    err = rel_l2(recs[False], g["rec"])
    assert err < 1e-5, f"rel-L2 {err:.3e}"
    if "rec_mute" in g:
        assert mute_consistent(g["rec"], g["rec_mute"], recs[True], recs[False])
