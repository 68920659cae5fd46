"""Known-answer tests of the oracle's restatement of AMRD's Berger-Oliger
MG-variable bookkeeping (oracle/bo_ops.c; amrd/evolve.c:344-366,
1621-1638, 1640-1700), with values worked out by hand from the
reference's formulas: the extrapolation coefficients of a coarse step and
of a fine sub-step, the TN method, the rotation of the extrapolation
levels with the eps_c correction and its net_rho per level (for L1 = 1 and
L1 > 1), and the brs copy."""
import ctypes as C

import numpy as np
import pytest

from oracle import portrun

D = C.POINTER(C.c_double)


@pytest.fixture(scope="module")
def lib():
    L = C.CDLL(portrun.build())
    L.oracle_mg_extrap.argtypes = [C.c_int] + [C.c_double] * 4 + [D] * 4 + [C.c_long]
    L.oracle_update_mg_extrap_vars.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int), C.c_int,
                                               C.POINTER(C.c_int), C.POINTER(D), C.POINTER(D),
                                               C.POINTER(D), C.POINTER(D), C.POINTER(C.c_long), C.c_double]
    L.oracle_set_mg_brs_vars.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(D),
                                         C.POINTER(D), C.POINTER(C.c_long)]
    return L


def _p(a):
    return a.ctypes.data_as(D)


def _pp(arrs):
    return (D * len(arrs))(*[_p(a) for a in arrs])


@pytest.mark.parametrize("tnp1,tnp1_lm1,dt_lm1,f1,f2", [
    (1.5, 1.5, 0.5, 2.0, -1.0),     # in step with the parent: linear extrapolation
    (1.25, 1.5, 0.5, 1.5, -0.5),    # first of two fine sub-steps
])
def test_extrap_from_etm1(lib, tnp1, tnp1_lm1, dt_lm1, f1, f2):
    e1 = np.array([3.0, -1.0, 0.25, 8.0])
    e2 = np.array([1.0, 2.0, -0.5, 4.0])
    out = np.zeros(4)
    assert lib.oracle_mg_extrap(0, tnp1, tnp1_lm1, 0.25, dt_lm1, _p(out), _p(np.zeros(4)), _p(e1), _p(e2), 4) == 0
    assert np.array_equal(out, f1 * e1 + f2 * e2)


def test_extrap_from_tn(lib):
    m1 = np.array([1.0, 2.0, 3.0])
    e1 = np.array([0.5, 0.5, 4.0])
    e2 = np.array([1.5, -0.5, 2.0])
    out = np.zeros(3)
    assert lib.oracle_mg_extrap(1, 0.0, 0.0, 0.25, 0.5, _p(out), _p(m1), _p(e1), _p(e2), 3) == 0
    assert np.array_equal(out, np.array([1.5, 1.5, 2.0]))   # m1 + 0.5 (e2 - e1)
    assert lib.oracle_mg_extrap(7, 0.0, 0.0, 0.25, 0.5, _p(out), _p(m1), _p(e1), _p(e2), 3) == 1


@pytest.mark.parametrize("L1,want", [
    # L1 = 1: net_rho 1, 2, 4 on levels 1..3 -> f = -, 1/2, 3/4; etm2 = 3 + 4 f
    (1, {1: 3.0, 2: 5.0, 3: 6.0}),
    # L1 = 2: levels 3.. only, net_rho starts at rho_tm[1] = 2 -> f = 1/2 on level 3
    (2, {1: 7.0, 2: 7.0, 3: 5.0}),
])
def test_update_rotates_and_corrects(lib, L1, want):
    levels = [1, 2, 3]
    e1 = [np.full(5, 3.0) for _ in levels]
    e2 = [np.full(5, 7.0) for _ in levels]
    m1 = [np.full(5, 5.0) for _ in levels]
    brs = [np.full(5, 1.0) for _ in levels]
    rho = (C.c_int * 4)(2, 2, 2, 2)
    lib.oracle_update_mg_extrap_vars(L1, 3, rho, 3, (C.c_int * 3)(*levels), _pp(e1), _pp(e2), _pp(m1), _pp(brs),
                                     (C.c_long * 3)(5, 5, 5), 1.0)
    for g, lev in enumerate(levels):
        assert np.all(e2[g] == want[lev]), (lev, e2[g])
        touched = lev >= L1 + (1 if L1 > 1 else 0)
        assert np.all(e1[g] == (5.0 if touched else 3.0))


def test_update_without_correction(lib):
    e1, e2, m1, brs = np.full(3, 2.0), np.full(3, 9.0), np.full(3, 6.0), np.zeros(3)
    rho = (C.c_int * 3)(2, 2, 2)
    lib.oracle_update_mg_extrap_vars(1, 2, rho, 1, (C.c_int * 1)(2), _pp([e1]), _pp([e2]), _pp([m1]), _pp([brs]),
                                     (C.c_long * 1)(3), 0.0)
    assert np.all(e2 == 2.0) and np.all(e1 == 6.0)


def test_set_brs_copies_the_levels_asked(lib):
    m1 = [np.arange(4.0) + 10 * g for g in range(3)]
    brs = [np.zeros(4) for _ in range(3)]
    lib.oracle_set_mg_brs_vars(2, 3, 3, (C.c_int * 3)(1, 2, 3), _pp(brs), _pp(m1), (C.c_long * 3)(4, 4, 4))
    assert not np.any(brs[0]) and np.array_equal(brs[1], m1[1]) and np.array_equal(brs[2], m1[2])
