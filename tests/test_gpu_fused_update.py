"""The mixed form's end-of-block kernel that carries the FP32 defect and
applies the update in one pass (its zeros go to the correction slot the
defect does not read, where the next block starts) gives the same solve,
bit for bit, as the separate defect and update kernels
(PGB_NO_FUSED_UPDATE=1): cycle count, per-cycle residuals and solution, for
every sweep kernel family that alternates the slots."""
import copy

import numpy as np
import pytest

from pamr_amrd_gb300 import workloads as W
from pamr_amrd_gb300.solver import Solver

pytestmark = pytest.mark.gpu

SWITCHES = ("PGB_NO_FUSED_UPDATE",)


def _run(monkeypatch, case, off, fuse):
    monkeypatch.setenv("PGB_SWEEP_FUSE", fuse)
    for v in SWITCHES:
        if v in off:
            monkeypatch.setenv(v, "1")
        else:
            monkeypatch.delenv(v, raising=False)
    s = Solver(copy.deepcopy(case))
    s.set_inputs()
    r = s.solve()
    u = s.get_u()
    s.close()
    return r["iters"], r["res"].copy(), u


@pytest.mark.parametrize("fuse", ["1", "2", "5", "6"])
@pytest.mark.parametrize("make", [lambda: W.conformal3d(65, 33, seed=2),
                                  lambda: W.poisson2d_uneven(seed=1, n=129, levels=5, min_boxes=8, max_boxes=24),
                                  lambda: W.lapse2d_bo(65, seed=2, levels=4),
                                  lambda: W.with_min_level(W.poisson2d_uneven(seed=7, n=129, levels=5, min_boxes=8,
                                                                              max_boxes=16), 3)],
                         ids=["c3d65", "uneven129", "lapse65", "uneven_min3"])
def test_fused_update_changes_no_bits(monkeypatch, make, fuse):
    case = make()
    case.params.precision = 1
    a = _run(monkeypatch, case, (), fuse)
    for off in (SWITCHES,):
        b = _run(monkeypatch, case, off, fuse)
        assert a[0] == b[0], off
        assert np.array_equal(a[1], b[1]), off
        for x, y in zip(a[2], b[2]):
            assert np.array_equal(x, y), off
    assert a[1][-1] <= case.params.tol
