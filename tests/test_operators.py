"""Level operators registered as expressions (pgb_operator_create): the
built-in PDEs are recognised as their compiled forms, malformed expressions
are errors, and a program evaluates with one IEEE rounding per operation in
the written order -- the order of the application hook it restates
(examples/nbs/num.f:113-116 for the nbs potential). No GPU needed."""
import ctypes as C

import numpy as np
import pytest

from pamr_amrd_gb300 import solver as S
from pamr_amrd_gb300 import workloads as W


def _eval(op, lap, j0, u, s):
    L, J = C.c_double(), C.c_double()
    sv = (C.c_double * 4)(*(list(s) + [0.0] * (4 - len(s))))
    S._check(S.lib().pgb_operator_eval(op.h, lap, j0, u, sv, C.byref(L), C.byref(J)))
    return L.value, J.value


def test_builtins_are_recognised():
    for pde in (W.POISSON, W.CONFORMAL, W.LAPSE):
        assert S.Operator(pde=pde).kind() == pde
    n, lop, jac = W.OPERATORS[W.NBS]
    assert S.Operator(nsrc=n, lop=lop, jac=jac).kind() == 3
    # the conformal operator written out is the built-in one
    op = S.Operator(nsrc=1, lop="lap + 6.283185307179586*s0*(((u*u)*(u*u))*u)",
                    jac="j0 + 31.41592653589793*s0*((u*u)*(u*u))")
    assert op.kind() == W.CONFORMAL


@pytest.mark.parametrize("lop,jac,nsrc", [
    ("lap - s1", "j0", 1),          # source beyond the count
    ("lap - ", "j0", 1),            # incomplete
    ("lap - s0)", "j0", 1),         # unbalanced
    ("j0 - s0", "j0", 1),           # j0 belongs to dL/du
    ("lap - s0", "lap", 1),         # lap belongs to L[u]
    ("lap - exp(s0)", "j0", 1),     # no functions
    ("lap" + " + u" * 40, "j0", 1), # too long
])
def test_malformed_expressions_are_errors(lop, jac, nsrc):
    with pytest.raises(S.PgbError):
        S.Operator(nsrc=nsrc, lop=lop, jac=jac)


def test_program_rounds_like_the_hook_order():
    """the nbs potential and the built-in operators, evaluated by the
    program on the host, equal numpy float64 in the hook's order bit for bit"""
    rng = np.random.default_rng(5)
    n, lop, jac = W.OPERATORS[W.NBS]
    nbs = S.Operator(nsrc=n, lop=lop, jac=jac)
    conf = S.Operator(pde=W.CONFORMAL)
    lapse = S.Operator(pde=W.LAPSE)
    for _ in range(2000):
        lap, j0, u, s0, s1 = (float(v) for v in rng.standard_normal(5) * 10.0 ** rng.integers(-6, 6, 5))
        L, J = _eval(nbs, lap, j0, u, [s0, s1])
        assert L == np.float64(lap) - (np.float64(s0) * s0 + np.float64(s1) * s1) and J == j0
        L, J = _eval(conf, lap, j0, u, [s0])
        p4 = (np.float64(u) * u) * (np.float64(u) * u)
        assert L == lap + 6.283185307179586 * np.float64(s0) * (p4 * u)
        assert J == j0 + 31.41592653589793 * np.float64(s0) * p4
        L, J = _eval(lapse, lap, j0, u, [s0])
        assert L == lap - np.float64(s0) * u and J == j0 - s0


def test_host_only_solver_takes_an_application_operator():
    """a hierarchy with the two-source nbs operator builds without a GPU and
    refuses a source index beyond the operator's count"""
    case = W.nbs2d_uneven(seed=3, n=33, levels=3, min_boxes=2, max_boxes=4, min_side=5, max_side=17)
    s = S.Solver(case, host_only=True)
    assert s.op_kind == 3
    assert s.num_levels() >= 3
    s.close()
