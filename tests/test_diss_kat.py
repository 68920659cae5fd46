"""Known-answer tests of the oracle's restatement of dmdiss3d
(src/m_util_r8.f:1690-1956), values worked out by hand from the Fortran:
a delta's 4th-difference footprint in the interior (-1, 4, -6, 4, -1)/16,
linear data untouched and quadratic data touched only where the one-sided
2nd difference applies, the even and odd parity variants at a physical
face, the mask, and the product of the three independent passes in 3-D."""
import ctypes as C

import numpy as np
import pytest

from oracle import portrun

D, I = C.POINTER(C.c_double), C.POINTER(C.c_int)
EVEN, ODD, OTHER = 3, 4, 0


@pytest.fixture(scope="module")
def lib():
    return C.CDLL(portrun.build())


def diss(lib, f, eps=0.5, do_bdy=0, pbt=(OTHER,) * 6, mask=None, shape=None):
    nx, ny, nz = shape or (f.size, 1, 1)
    f = np.ascontiguousarray(f, dtype=np.float64).copy()
    work = np.zeros_like(f)
    mask = np.ones_like(f) if mask is None else np.ascontiguousarray(mask, dtype=np.float64)
    e, mo = np.array([eps]), C.c_double(0.0)
    ci = lambda v: C.byref(C.c_int(v))  # noqa: E731
    lib.dmdiss3d_(f.ctypes.data_as(D), work.ctypes.data_as(D), e.ctypes.data_as(D), ci(do_bdy),
                  (C.c_int * 6)(*pbt), ci(EVEN), ci(ODD), mask.ctypes.data_as(D), C.byref(mo), ci(nx), ci(ny),
                  ci(nz), e.ctypes.data_as(D), C.byref(C.c_double(0.0)), ci(0))
    return f, work


def test_interior_delta(lib):
    f = np.zeros(9)
    f[4] = 1.0
    out, work = diss(lib, f)
    want = np.zeros(9)
    want[2:7] = -0.5 * np.array([1, -4, 6, -4, 1]) / 16
    want[4] += 1
    assert np.array_equal(out, want)
    assert np.array_equal(work, f)   # work holds the last pass's input


def test_linear_is_untouched_and_quadratic_only_at_the_ends(lib):
    x = np.arange(1.0, 10.0)
    out, _ = diss(lib, 3 * x - 2, do_bdy=1)
    assert np.array_equal(out, 3 * x - 2)
    out, _ = diss(lib, x * x, do_bdy=1)
    want = x * x
    want[[0, -1]] -= 0.5 * 0.25 * 2   # w2 (f1 - 2 f2 + f3) = 2/4
    assert np.array_equal(out, want)  # 4th and one-sided 3rd differences of x^2 vanish


@pytest.mark.parametrize("pbt,f2", [(EVEN, 1 - 0.5 * 7 / 16), (ODD, 1 - 0.5 * 5 / 16)])
def test_parity_at_the_lower_face(lib, pbt, f2):
    f = np.zeros(9)
    f[1] = 1.0                        # delta at i = 2
    out, _ = diss(lib, f, pbt=(pbt,) + (OTHER,) * 5)
    assert out[1] == f2               # (+-f(i)) + f(i+2) - 4 (f(i-1) + f(i+1)) + 6 f(i) = 7 or 5
    # at i = 1 the reflection doubles the neighbour: -4 ((+-f(2)) + f(2)) = -8 (even) or 0 (odd)
    assert out[0] == (0.5 * 8 / 16 if pbt == EVEN else 0.0)


def test_mask_off_points_keep_their_value(lib):
    f = np.zeros(9)
    f[4] = 1.0
    mask = np.ones(9)
    mask[[3, 4]] = 0.0
    out, _ = diss(lib, f, mask=mask)
    assert out[3] == 0.0 and out[4] == 1.0 and out[5] == 0.5 * 4 / 16


def test_three_passes_multiply(lib):
    n = 7
    f = np.zeros((n, n, n))
    f[3, 3, 3] = 1.0
    out, _ = diss(lib, f.reshape(-1), shape=(n, n, n))
    assert out.reshape(n, n, n)[3, 3, 3] == (13 / 16) ** 3


def diss_ex(lib, f, chr_, eps=0.5, do_bdy=1, pbt=(OTHER,) * 6, do_ex=1, shape=None, ex=-1.0, mask=None):
    nx, ny, nz = shape or (f.size, 1, 1)
    f = np.ascontiguousarray(f, dtype=np.float64).copy()
    work = np.zeros_like(f)
    mask = np.ones_like(f) if mask is None else np.ascontiguousarray(mask, dtype=np.float64)
    e = np.ascontiguousarray(np.atleast_1d(eps), dtype=np.float64)
    c = np.ascontiguousarray(chr_, dtype=np.float64)
    ci = lambda v: C.byref(C.c_int(v))  # noqa: E731
    lib.dmdiss3d_(f.ctypes.data_as(D), work.ctypes.data_as(D), e.ctypes.data_as(D), ci(do_bdy),
                  (C.c_int * 6)(*pbt), ci(EVEN), ci(ODD), mask.ctypes.data_as(D), C.byref(C.c_double(0.0)),
                  ci(nx), ci(ny), ci(nz), c.ctypes.data_as(D), C.byref(C.c_double(ex)), ci(do_ex))
    return f


@pytest.mark.parametrize("pbt", [(OTHER,) * 6, (EVEN, ODD, ODD, EVEN, OTHER, EVEN)])
def test_excised_path_without_excision_equals_the_plain_path(lib, pbt):
    """with no excised point, do_bdy = 1 and lines of 5 or more, the
    excised branches reduce to the plain ones (same stencils, same order)"""
    rng = np.random.default_rng(5)
    shape = (9, 7, 6)
    f = rng.standard_normal(int(np.prod(shape)))
    plain, _ = diss(lib, f, do_bdy=1, pbt=pbt, shape=shape)
    ex = diss_ex(lib, f, np.zeros_like(f), do_bdy=1, pbt=pbt, shape=shape)
    assert np.array_equal(plain, ex)


def test_one_sided_next_to_an_excised_point(lib):
    f = np.zeros(11)
    f[5] = 1.0                        # i = 6
    chr_ = np.zeros(11)
    chr_[6] = -1.0                    # i = 7 excised
    out = diss_ex(lib, f, chr_, do_bdy=1)
    assert out[6] == 0.0              # the excised point is left alone
    assert out[5] == 1 - 0.5 * 0.25   # i = 6: w2 (f(i) - 2 f(i-1) + f(i-2)) = 1/4
    # i = 5: X(+2) fails, so the one-sided 3rd difference towards the left: w3 (-f(i+1) + 3 f(i) - 3 f(i-1) + f(i-2))
    assert out[4] == -0.5 * (1 / 8) * (-1.0)


def test_do_bdy_zero_keeps_only_the_end_rule(lib):
    f = np.zeros(11)
    f[5] = 1.0
    chr_ = np.zeros(11)
    chr_[6] = -1.0
    out = diss_ex(lib, f, chr_, do_bdy=0)
    assert out[5] == 1.0 and out[4] == 0.0   # one-sided branches off with do_bdy = 0
    chr_ = np.zeros(11)
    chr_[0] = -1.0                            # i = 1 excised: i = 2 takes w2 towards the right
    g = np.zeros(11)
    g[1] = 1.0
    out = diss_ex(lib, g, chr_, do_bdy=0)
    assert out[1] == 1 - 0.5 * 0.25


def test_per_point_eps_with_negative_do_ex(lib):
    f = np.zeros(9)
    f[4] = 1.0
    eps = np.full(9, 0.5)
    eps[4] = 0.25
    out = diss_ex(lib, f, np.zeros(9), eps=eps, do_ex=-1)
    assert out[4] == 1 - 0.25 * 6 / 16 and out[3] == 0.5 * 4 / 16
