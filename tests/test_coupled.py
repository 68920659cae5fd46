"""Several elliptic variables on the host side (no GPU): the operator
programs name the other variables as u0..u3 and round like the hook
formulas of the coupled pair (oracle/mg_ops.c: L_u = lap u - s0*(u - w) -
s1, L_w = lap w - s0*(w - u), both with diagonal j0 - s0); a program naming
a variable the solver lacks is refused; both forms take several variables;
the hierarchy and plans build for them."""
import ctypes as C

import numpy as np
import pytest

from pamr_amrd_gb300 import solver as S
from pamr_amrd_gb300 import workloads as W


def _eval(op, var, lap, j0, uv, s):
    L, J = C.c_double(), C.c_double()
    u4 = (C.c_double * 4)(*(list(uv) + [0.0] * (4 - len(uv))))
    s4 = (C.c_double * 4)(*(list(s) + [0.0] * (4 - len(s))))
    S.lib().pgb_operator_eval_vars.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double,
                                               C.POINTER(C.c_double), C.POINTER(C.c_double),
                                               C.POINTER(C.c_double), C.POINTER(C.c_double)]
    S._check(S.lib().pgb_operator_eval_vars(op.h, var, lap, j0, u4, s4, C.byref(L), C.byref(J)))
    return L.value, J.value


def test_coupled_programs_round_like_the_hooks():
    rng = np.random.default_rng(5)
    nsrc, pairs = W.VAR_OPERATORS[W.COUPLED]
    ops = [S.Operator(nsrc=nsrc, lop=l, jac=j) for l, j in pairs]
    for _ in range(200):
        lap, j0, u, w, s0, s1 = (float(x) for x in rng.standard_normal(6) * 10.0 ** rng.integers(-3, 4, 6))
        Lu, Ju = _eval(ops[0], 0, lap, j0, [u, w], [s0, s1])
        Lw, Jw = _eval(ops[1], 1, lap, j0, [u, w], [s0, s1])
        assert Lu == lap - s0 * (u - w) - s1 and Ju == j0 - s0
        assert Lw == lap - s0 * (w - u) and Jw == j0 - s0


def test_program_naming_a_missing_variable_is_refused():
    case = W.poisson2d(17, seed=0)
    op = S.Operator(nsrc=1, lop="lap - s0*u1", jac="j0")
    with pytest.raises(S.PgbError):
        S.Solver(case, host_only=True, op=op)


def test_mixed_form_takes_several_variables():
    case = W.coupled_from(W.poisson2d(17, seed=0), seed=1)
    case.params.precision = 1
    s = S.Solver(case, host_only=True)
    assert s.num_levels() >= 2
    s.close()


def test_two_variable_hierarchy_builds_its_plans():
    case = W.coupled_from(W.poisson2d_uneven(seed=1, n=33, levels=3, min_boxes=2, max_boxes=4, min_side=5,
                                             max_side=17), seed=3)
    s = S.Solver(case, host_only=True)
    one = S.Solver(W.poisson2d_uneven(seed=1, n=33, levels=3, min_boxes=2, max_boxes=4, min_side=5,
                                      max_side=17), host_only=True)
    assert s.num_levels() == one.num_levels()
    for L in range(1, s.num_levels() + 1):   # the same transfer lists as one variable
        for which in (0, 3, 5):
            assert np.array_equal(s.plan(which, L)[:, :14], one.plan(which, L)[:, :14])
    s.close()
    one.close()


@pytest.mark.parametrize("lop,fixed", [("lap - s0*(u - u1) - s1", 1), ("lap - s0*(u - u0)", 1),
                                       ("lap - u1/s0 + 2*s1", 1), ("lap - s0*u*u1", 0),
                                       ("lap - s0/u1", 0), ("lap*u1", 0), ("lap - (u1 + s0)*(u1 - s0)", 0)])
def test_fixed_coupling_coefficients_are_recognised(lop, fixed):
    """the mixed form computes dL/du_k once per prepare only where no such
    derivative of the program depends on lap or a variable"""
    op = S.Operator(nsrc=2, lop=lop, jac="j0")
    S.lib().pgb_operator_device_form.restype = C.c_void_p
    S.lib().pgb_operator_device_form.argtypes = [C.c_void_p]
    S.lib().pgb_dop_couplings_fixed.argtypes = [C.c_void_p]
    assert S.lib().pgb_dop_couplings_fixed(S.lib().pgb_operator_device_form(op.h)) == fixed


@pytest.mark.parametrize("jac,fixed", [("j0 - s0", 1), ("j0", 1), ("j0 - s0*s1 + 3", 1), ("j0 - s0*u1", 0),
                                       ("j0 + 5*u*u*u*u", 0)])
def test_fixed_jacobian_terms_are_recognised(jac, fixed):
    """likewise the Jacobian term dL/du - j0: once per prepare where the dL/du
    program reads no variable (nor lap)"""
    op = S.Operator(nsrc=2, lop="lap - s0*(u - u1) - s1", jac=jac)
    S.lib().pgb_operator_device_form.restype = C.c_void_p
    S.lib().pgb_operator_device_form.argtypes = [C.c_void_p]
    S.lib().pgb_dop_jac_fixed.argtypes = [C.c_void_p]
    assert S.lib().pgb_dop_jac_fixed(S.lib().pgb_operator_device_form(op.h)) == fixed
