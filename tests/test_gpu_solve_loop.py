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


def _run(monkeypatch, case, host_loop):
    if host_loop:
        monkeypatch.setenv("PGB_HOST_LOOP", "1")
    else:
        monkeypatch.delenv("PGB_HOST_LOOP", raising=False)
    s = Solver(case)
    out = []
    for _ in range(2):
        s.set_inputs()
        r = s.solve()
        out.append((r["iters"], r["res"].copy(), r["res_final"], s.get_u()))
    s.close()
    return out


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
@pytest.mark.parametrize("limits", [None, ("max_iter", 3), ("min_iter", 30)],
                         ids=["tol", "max_iter3", "min_iter30"])
def test_device_loop_equals_host_loop(monkeypatch, precision, limits):
    case = copy.deepcopy(W.conformal3d(65, 33, seed=2))
    case.params.precision = precision
    if limits:
        setattr(case.params, limits[0], limits[1])
    dev = _run(monkeypatch, case, False)
    host = _run(monkeypatch, case, True)
    for (i1, r1, f1, u1), (i2, r2, f2, u2) in zip(dev, host):
        assert i1 == i2
        if limits and limits[0] == "max_iter":
            assert i1 == 3
        if limits and limits[0] == "min_iter":
            assert i1 >= 30
        assert np.array_equal(r1, r2)
        assert f1 == f2
        for a, b in zip(u1, u2):
            assert np.array_equal(a, b)
