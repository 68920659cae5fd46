"""The drop-in multigrid module on the GPU: an nbs-style AMRD application
(tests/dropin/nbs_app.c) calls the reference's entry points
solve_elliptics / vcycle (amrd/mg.h:32-37) of libamrd_mg_gb300 over a PAMR
environment, and reproduces what the same application source computes with
the reference's own PAMR/AMRD and amrd/mg.c (golden fixtures): the same
cycle count, u bit-identical and the same cmask on every AMR grid, and the
finest residual of every cycle within 1e-12 relative (only the norm's
summation order differs). Mode 1 is the evolution iteration's pattern: an
MG hierarchy of the finest level and single vcycle calls with the sources
changed between them (amrd/evolve.c:454-493). Coupled cases solve two
elliptic variables together (both registered for the device, both compared
bit for bit)."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "dropin"))
import dropin as D  # noqa: E402
import golden_cases as G  # noqa: E402

pytestmark = pytest.mark.gpu

NORM_RTOL = 1e-12
ERR_RTOL = 1e-9


@pytest.mark.parametrize("path", G.dropin_files(), ids=lambda p: os.path.basename(p)[7:-4])
def test_application_through_the_drop_in_matches_reference(path):
    case, mode, arg, level, ref = G.load_dropin(path)
    out = D.run(D.build_device_app(), case, mode, arg, level)
    assert out["iters"] == ref["iters"]
    assert len(out["grids"]) == len(ref["grids"])
    for a, b in zip(out["grids"], ref["grids"]):
        assert a["level"] == b["level"] and a["shape"] == b["shape"]
        assert np.array_equal(a["u"], b["u"])
        assert np.array_equal(a["cmask"], b["cmask"])
        if "w" in b:   # the second elliptic variable of a coupled case
            assert np.array_equal(a["w"], b["w"])
    assert len(out["res"]) == len(ref["res"])
    assert float(np.max(np.abs(out["res"] - ref["res"]) / np.abs(ref["res"]))) < NORM_RTOL


@pytest.mark.parametrize("path", [p for p in G.dropin_files() if "_m0_" in p],
                         ids=lambda p: os.path.basename(p)[7:-4])
def test_application_mixed_precision_through_the_drop_in(path):
    """amrd_set_device_MG_precision(1): FP32 smoothing inside FP64 defect
    correction, converged and within 1e-9 of the reference's solution (both
    elliptic variables of a coupled case)"""
    case, mode, arg, level, ref = G.load_dropin(path)
    if ref["res"][-1] > case.params.tol:
        pytest.skip("the reference did not reach its tolerance on this case")
    out = D.run(D.build_device_app(), case, mode, arg, level, env={"NBS_APP_MIXED": "1"})
    assert out["res"][-1] <= case.params.tol
    for f in ("u", "w"):
        if f not in ref["grids"][0]:
            continue
        umax = max(float(np.max(np.abs(g[f]))) for g in ref["grids"])
        err = max(float(np.max(np.abs(a[f] - b[f]))) for a, b in zip(out["grids"], ref["grids"]))
        assert err <= ERR_RTOL * umax, (f, err / umax)
