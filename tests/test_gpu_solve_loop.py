"""The device-resident solve loop (a CUDA-graph conditional while node
around the captured V-cycle) against the host loop (PGB_HOST_LOOP=1): same
cycle count, same per-cycle residuals and the same solution bit for bit,
including a solve stopped by max_iter and one held on by min_iter."""
import copy

import numpy as np
import pytest

from pamr_amrd_gb300 import workloads as W
from pamr_amrd_gb300.solver import Solver

pytestmark = pytest.mark.gpu


def _solve(monkeypatch, s, host_loop):
    if host_loop:
        monkeypatch.setenv("PGB_HOST_LOOP", "1")
    else:
        monkeypatch.delenv("PGB_HOST_LOOP", raising=False)
    s.set_inputs()
    r = s.solve()
    return r["iters"], r["res"].copy(), r["res_final"], s.get_u()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
@pytest.mark.parametrize("limits", [None, ("max_iter", 3), ("min_iter", 30)],
                         ids=["tol", "max_iter3", "min_iter30"])
def test_device_loop_equals_host_loop(monkeypatch, precision, limits):
    case = copy.deepcopy(W.conformal3d(65, 33, seed=2))
    case.params.precision = precision
    if limits:
        setattr(case.params, limits[0], limits[1])
    # one solver for both loops: the mixed form's autotuner picks tile depths
    # per solver, and a different depth moves the FP32/FP64 split a little
    s = Solver(case)
    runs = [(_solve(monkeypatch, s, False), _solve(monkeypatch, s, True)) for _ in range(2)]
    s.close()
    for (i1, r1, f1, u1), (i2, r2, f2, u2) in runs:
        assert i1 == i2
        if limits and limits[0] == "max_iter":
            assert i1 == 3
        if limits and limits[0] == "min_iter":
            assert i1 >= 30
        assert np.array_equal(r1, r2)
        assert f1 == f2
        for a, b in zip(u1, u2):
            assert np.array_equal(a, b)
