"""Registered level operators and MG hierarchies built from an AMR level
above the base, on the GPU through the C ABI.

* The operator program (pgb_op.cuh) against the compiled built-in forms:
  PGB_OP_INTERPRET=1 evaluates the built-in PDEs through their programs;
  the FP64 solve must not change by a bit.
* The nbs potential (examples/nbs/num.f:85-246, two sources), an operator
  the library does not build in: bit-identical to the oracle port beyond
  the golden fixtures (which test_gpu_parity.py covers against the compiled
  reference), and within 1e-9 in the mixed form.
* min_level (PAMR_build_mgh(min_lev, ...), src/gh.c:1222): the hierarchy of
  solve_elliptics(L > 1) and of the evolution iteration's V-cycle
  (amrd/evolve.c:454-483, finest level only), bit-identical to the port,
  and single V-cycles (pgb_vcycle, the vcycle of amrd/evolve.c:483) equal
  the port's cycles one by one.
"""
import copy

import numpy as np
import pytest

from oracle import portrun
from pamr_amrd_gb300 import workloads as W
from pamr_amrd_gb300.solver import Solver

pytestmark = pytest.mark.gpu

NORM_RTOL = 1e-12
ERR_RTOL = 1e-9


def _solve(case, trace=0):
    s = Solver(case)
    s.set_inputs()
    if trace:
        s.trace_enable(trace)
    r = s.solve()
    r["u"] = s.get_u()
    if trace:
        r["trace"] = s.trace_fetch()
    r["kind"] = s.op_kind
    s.close()
    return r


@pytest.mark.parametrize("make", [lambda: W.conformal3d(33, 17, seed=4),
                                  lambda: W.lapse2d_bo(65, seed=6, levels=4, step=50),
                                  lambda: W.poisson2d_uneven(seed=8, n=65, levels=4, min_boxes=4,
                                                             max_boxes=10)],
                         ids=["conformal", "lapse", "poisson_uneven"])
def test_program_form_equals_compiled_builtin(make, monkeypatch):
    a = _solve(make(), trace=100000)
    monkeypatch.setenv("PGB_OP_INTERPRET", "1")
    b = _solve(make(), trace=100000)
    assert a["kind"] != 3 and b["kind"] == 3
    assert a["iters"] == b["iters"]
    for x, y in zip(a["u"], b["u"]):
        assert np.array_equal(x, y)
    assert np.array_equal(a["trace"]["norm"], b["trace"]["norm"])


NBS = [lambda: W.nbs3d(33, 17, seed=1),
       lambda: W.nbs3d(65, 33, seed=2, levels=3),
       lambda: W.nbs2d_uneven(seed=4),
       lambda: W.nbs2d_uneven(seed=5, n=129, levels=5, min_boxes=8, max_boxes=24, min_side=17,
                              max_side=65)]
NBS_IDS = ["nbs3d33", "nbs3d65_L3", "nbs2d_uneven65", "nbs2d_uneven129"]


@pytest.mark.parametrize("make", NBS, ids=NBS_IDS)
def test_nbs_operator_matches_port(make):
    case = make()
    r = _solve(case)
    assert r["kind"] == 3
    p = portrun.solve(case)
    assert r["iters"] == p["iters"]
    for a, b in zip(r["u"], p["u"]):
        assert np.array_equal(a, b)
    assert np.max(np.abs(r["res"] - p["res"]) / p["res"]) < NORM_RTOL
    assert r["res_final"] <= case.params.tol


@pytest.mark.parametrize("make", NBS[:3], ids=NBS_IDS[:3])
def test_nbs_operator_mixed_form(make):
    case = make()
    p = portrun.solve(case)
    c = copy.deepcopy(case)
    c.params.precision = 1
    r = _solve(c)
    assert r["res_final"] <= case.params.tol
    umax = max(float(np.max(np.abs(a))) for a in p["u"])
    err = max(float(np.max(np.abs(a - b))) for a, b in zip(r["u"], p["u"]))
    assert err <= ERR_RTOL * umax, err / umax
    assert abs(r["iters"] - p["iters"]) <= 2


MINL = [(lambda: W.lapse2d_bo(65, seed=6, levels=4, step=90), 2),
        (lambda: W.lapse2d_bo(65, seed=6, levels=4, step=90), 3),
        (lambda: W.lapse2d_bo(65, seed=6, levels=4, step=90), 4),
        (lambda: W.poisson2d_uneven(seed=7, n=129, levels=5, min_boxes=8, max_boxes=16), 3),
        (lambda: W.conformal3d(65, 33, seed=5), 2),
        (lambda: W.nbs3d(33, 17, seed=3, levels=3), 3)]
MINL_IDS = ["lapse_min2", "lapse_min3", "lapse_min4", "uneven_min3", "conformal_min2", "nbs_min3"]


@pytest.mark.parametrize("make,level", MINL, ids=MINL_IDS)
def test_min_level_hierarchy_matches_port(make, level):
    case = W.with_min_level(make(), level)
    r = _solve(case)
    p = portrun.solve(case)
    assert r["iters"] == p["iters"]
    for a, b in zip(r["u"], p["u"]):
        assert np.array_equal(a, b)
    assert np.max(np.abs(r["res"] - p["res"]) / p["res"]) < NORM_RTOL


@pytest.mark.parametrize("make,level", MINL[1:3] + MINL[3:4], ids=MINL_IDS[1:3] + MINL_IDS[3:4])
def test_min_level_mixed_form(make, level):
    case = W.with_min_level(make(), level)
    p = portrun.solve(case)
    c = copy.deepcopy(case)
    c.params.precision = 1
    r = _solve(c)
    assert r["res_final"] <= case.params.tol
    umax = max(float(np.max(np.abs(a))) for a in p["u"])
    err = max(float(np.max(np.abs(a - b))) for a, b in zip(r["u"], p["u"]))
    assert err <= ERR_RTOL * umax, err / umax


def test_single_vcycles_on_the_finest_level_hierarchy():
    """the evolution iteration's pattern: PAMR_build_mgh(Lf, Lf, 1) then one
    vcycle per iteration (amrd/evolve.c:454-483). k calls of pgb_vcycle on a
    min_level = Lf hierarchy equal k cycles of the port, cycle for cycle."""
    case = W.with_min_level(W.lapse2d_bo(65, seed=9, levels=4, step=10), 4)
    k = 5
    s = Solver(case)
    s.set_inputs()
    res = [s.vcycle() for _ in range(k)]
    u = s.get_u()
    s.close()
    c = copy.deepcopy(case)
    c.params.max_iter = c.params.min_iter = k
    c.params.tol = 0.0
    p = portrun.solve(c)
    assert p["iters"] == k
    assert np.max(np.abs(np.array(res) - p["res"]) / p["res"]) < NORM_RTOL
    for a, b in zip(u, p["u"]):
        assert np.array_equal(a, b)
