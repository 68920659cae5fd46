"""Failure handling without any GPU fault: non-convergence is reported as a
status, NaN input ends the solve instead of hanging, bad calls return error
codes and leave the context usable."""
import numpy as np
import pytest

from pamr_amrd_gb300 import workloads as W
from pamr_amrd_gb300.solver import PgbError, Solver, lib

pytestmark = pytest.mark.gpu


def test_forced_non_convergence_returns_status():
    case = W.poisson2d(65)
    case.params.max_iter = 1
    s = Solver(case)
    s.set_inputs()
    r = s.solve()
    assert r["iters"] == 1 and r["res_final"] > case.params.tol


def test_nan_input_terminates():
    case = W.poisson2d(33)
    case.params.max_iter = 3
    case.src[0][100] = np.nan
    s = Solver(case)
    s.set_inputs()
    r = s.solve()
    assert r["iters"] <= 3 and not np.isfinite(r["res_final"])
    # the context is still usable afterwards
    ok = W.poisson2d(17)
    s2 = Solver(ok)
    s2.set_inputs()
    assert s2.solve()["res_final"] <= ok.params.tol


def test_bad_grid_index_is_an_error():
    s = Solver(W.poisson2d(17))
    with pytest.raises(PgbError):
        s.get_u.__func__  # noqa: B018
        import ctypes as C
        a = np.zeros(17 * 17)
        rc = lib().pgb_get_grid(s.h, 5, a.ctypes.data_as(C.POINTER(C.c_double)))
        if rc:
            raise PgbError(lib().pgb_last_error().decode())
