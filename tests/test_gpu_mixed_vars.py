"""Several elliptic variables in the mixed form (FP32 smoothing and
prolongation inside FP64 defect correction; each variable's FP64 passes run
over its view of the boxes, the coupled FP32 smoother relaxes every
variable's correction point by point with coupling coefficients from the
programs' derivatives): the coupled pair (workloads.VAR_OPERATORS[COUPLED])
converges to the relative residual the FP64 form reaches in the same number
of V-cycles (within one), also where the coupling s0 dx^2 is large on the
coarse levels, and both variables agree with the FP64 solution, which is
bit-identical to the compiled reference's (test_gpu_coupled.py), within 1e-9
of max |u| on every grid. The golden cases the reference solved to its
tolerance agree with its own solution the same way."""
import copy

import numpy as np
import pytest

import golden_cases as G
from pamr_amrd_gb300 import workloads as W
from pamr_amrd_gb300.solver import Solver

pytestmark = pytest.mark.gpu

ERR_RTOL = 1e-9

CASES = {
    "p2d129": lambda: W.coupled_from(W.poisson2d(129, seed=2), seed=3),
    "c3d65": lambda: W.coupled_from(W.conformal3d(65, 33, seed=1), seed=2),
    "uneven129": lambda: W.coupled_from(W.poisson2d_uneven(seed=2, n=129, levels=4, min_boxes=4, max_boxes=8),
                                        seed=4),
    "nbs3d33": lambda: W.coupled_from(W.nbs3d(33, 17, seed=1), seed=5),
    "p3d65": lambda: W.coupled_from(W.poisson3d(65, seed=1), seed=2),
    "c3d129": lambda: W.coupled_from(W.conformal3d(129, 65, seed=0), seed=1),
}


def _solve(case, precision, monkeypatch=None, env=None):
    c = copy.deepcopy(case)
    c.params.precision = precision
    for k, v in (env or {}).items():
        monkeypatch.setenv(k, v)
    try:
        s = Solver(c)
        s.set_inputs()
        r = s.solve()
        r["vars"] = s.get_vars()
        s.close()
    finally:
        for k in env or {}:
            monkeypatch.delenv(k)
    return r


def _close(got, ref):
    for v, (a, b) in enumerate(zip(got, ref)):
        umax = max(float(np.max(np.abs(x))) for x in b)
        err = max(float(np.max(np.abs(x - y))) for x, y in zip(a, b))
        assert err <= ERR_RTOL * umax, (v, err / umax)


@pytest.mark.parametrize("name", list(CASES))
def test_mixed_several_variables_match_the_fp64_form(name):
    case = CASES[name]()
    mixed, fp64 = _solve(case, 1), _solve(case, 0)
    assert fp64["res_final"] <= case.params.tol
    assert mixed["res_final"] <= case.params.tol
    assert abs(mixed["iters"] - fp64["iters"]) <= 1, (mixed["iters"], fp64["iters"])
    _close(mixed["vars"], fp64["vars"])


@pytest.mark.parametrize("path", G.coupled_files(), ids=lambda p: p.split("/")[-1][:-4])
def test_mixed_several_variables_match_reference_fixture(path):
    case, ref = G.load(path)
    if ref["iters"] >= case.params.max_iter:
        pytest.skip("the reference ran this case to max_iter, not to its tolerance")
    r = _solve(case, 1)
    assert r["res_final"] <= case.params.tol
    _close(r["vars"], [ref["u"], ref["u_extra"][0]])


def test_mixed_several_variables_same_bits_in_every_launch_mode(monkeypatch):
    """the device solve loop, the host loop over captured cycles and direct
    launches run the same kernels in the same order"""
    case = CASES["uneven129"]()
    ref = _solve(case, 1, monkeypatch, {"PGB_AUTOTUNE": "0"})
    for env in ({"PGB_HOST_LOOP": "1"}, {"PGB_NO_GRAPH": "1", "PGB_HOST_LOOP": "1"}):
        r = _solve(case, 1, monkeypatch, dict(env, PGB_AUTOTUNE="0"))
        assert r["iters"] == ref["iters"] and r["res_final"] == ref["res_final"]
        for a, b in zip(r["vars"], ref["vars"]):
            for x, y in zip(a, b):
                assert np.array_equal(x, y)


def test_fixed_couplings_once_per_prepare_change_no_bits(monkeypatch):
    """the coupled pair's coefficients dL/du_k and Jacobian terms are sources
    only: computed once per prepare (the default) or in every FP64 pass
    (PGB_COUPLINGS_EVERY_PASS=1), the solve is the same bit for bit"""
    case = CASES["c3d65"]()
    ref = _solve(case, 1, monkeypatch, {"PGB_AUTOTUNE": "0", "PGB_COUPLINGS_EVERY_PASS": "1"})
    r = _solve(case, 1, monkeypatch, {"PGB_AUTOTUNE": "0"})
    assert r["iters"] == ref["iters"] and r["res_final"] == ref["res_final"]
    for a, b in zip(r["vars"], ref["vars"]):
        for x, y in zip(a, b):
            assert np.array_equal(x, y)
