"""Known-answer tests of the C restatement of src/m_util_r8.f the oracle
uses: interpolation is exact on polynomials of its order, half/full
weighting reproduce constants and linear functions, strided copy injects."""
import ctypes as C

import numpy as np
import pytest

from oracle import portrun


def _lib():
    return C.CDLL(portrun.build())


def _ip(v):
    return C.byref(C.c_int(int(v)))


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def interp(u1, shape1, ni, nj, nk, rho, ord_):
    L = _lib()
    n2 = [(ni - 1) * rho + 1, (nj - 1) * rho + 1, (nk - 1) * rho + 1 if nk > 1 else 1]
    u2 = np.zeros(n2[0] * n2[1] * n2[2])
    args = [*shape1, *n2, 1, 1, 1, 1, 1, 1, ni, nj, nk, 1, 1, 1, rho, rho, rho, ord_]
    ex = C.c_double(0)
    L.dminterp3d_(_dp(u1), _dp(u2), *[_ip(v) for v in args], _dp(u1), C.byref(ex), _ip(0))
    return u2.reshape(n2[2], n2[1], n2[0])


@pytest.mark.parametrize("ord_,deg", [(2, 1), (4, 3)])
def test_interp_exact_on_polynomials(ord_, deg):
    n = 9
    x = np.linspace(-1, 1, n)
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    f = lambda a, b, c: 0.3 + a ** deg - 0.5 * b ** deg + 0.25 * c * a ** (deg - 1)  # noqa: E731
    u1 = np.ascontiguousarray(f(X, Y, Z).transpose(2, 1, 0)).reshape(-1)
    out = interp(u1, (n, n, n), n, n, n, 2, ord_)
    xf = np.linspace(-1, 1, 2 * n - 1)
    Xf, Yf, Zf = np.meshgrid(xf, xf, xf, indexing="ij")
    want = f(Xf, Yf, Zf).transpose(2, 1, 0)
    assert np.max(np.abs(out - want)) < 1e-13


@pytest.mark.parametrize("fn", ["dmhwr3d_", "dmfwr3d_"])
def test_restriction_reproduces_linear(fn):
    L = _lib()
    n1, n2 = 17, 9
    x = np.linspace(0, 1, n1)
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    u1 = np.ascontiguousarray((1 + 2 * X - Y + 0.5 * Z).transpose(2, 1, 0)).reshape(-1)
    u2 = np.zeros(n2 ** 3)
    args = [n1, n1, n1, n2, n2, n2, 1, 1, 1, 1, 1, 1, n2, n2, n2, 2, 2, 2, 1, 1, 1]
    ex = C.c_double(0)
    getattr(L, fn)(_dp(u1), _dp(u2), *[_ip(v) for v in args], _dp(u1), C.byref(ex), _ip(0))
    xc = np.linspace(0, 1, n2)
    Xc, Yc, Zc = np.meshgrid(xc, xc, xc, indexing="ij")
    want = (1 + 2 * Xc - Yc + 0.5 * Zc).transpose(2, 1, 0).reshape(-1)
    assert np.max(np.abs(u2 - want)) < 1e-14


def test_strided_copy_is_straight_injection():
    L = _lib()
    n1, n2 = 9, 5
    u1 = np.arange(n1 * n1, dtype=np.float64)
    u2 = np.zeros(n2 * n2)
    args = [n1, n1, 1, n2, n2, 1, 1, 1, 1, 1, 1, 1, n2, n2, 1, 2, 2, 1, 1, 1, 1]
    L.dmcopy3d_(_dp(u1), _dp(u2), *[_ip(v) for v in args])
    assert np.array_equal(u2.reshape(n2, n2), u1.reshape(n1, n1)[::2, ::2])


# ------------------------------------------------------ excision (do_ex=1) --
EX = 1.0


def _ball_mask(n, centre, radius):
    x = np.arange(n)
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    inside = (X - centre[0]) ** 2 + (Y - centre[1]) ** 2 + (Z - centre[2]) ** 2 <= radius ** 2
    return np.ascontiguousarray(np.where(inside, EX, 0.0).transpose(2, 1, 0)).reshape(-1)


@pytest.mark.parametrize("fn", ["dmhwr3d_", "dmfwr3d_"])
def test_excised_restriction_of_constant(fn):
    """with excision a constant restricts to itself on unexcised points and to
    0 on excised ones (the weights renormalise over unexcised neighbours)"""
    L = _lib()
    n1, n2 = 17, 9
    u1 = np.full(n1 ** 3, 2.5)
    chr1 = _ball_mask(n1, (8, 9, 7), 4.2)
    u2 = np.full(n2 ** 3, -7.0)
    args = [n1, n1, n1, n2, n2, n2, 1, 1, 1, 1, 1, 1, n2, n2, n2, 2, 2, 2, 1, 1, 1]
    ex = C.c_double(EX)
    getattr(L, fn)(_dp(u1), _dp(u2), *[_ip(v) for v in args], _dp(chr1), C.byref(ex), _ip(1))
    fine_ex = chr1.reshape(n1, n1, n1)[::2, ::2, ::2].reshape(-1) == EX
    assert np.all(u2[fine_ex] == 0.0)
    assert np.max(np.abs(u2[~fine_ex] - 2.5)) < 1e-14


@pytest.mark.parametrize("ord_", [2, 4])
def test_excised_interp_of_linear_away_from_the_hole(ord_):
    """values inside the excised ball are garbage; fine points whose coarse
    stencil never touches it interpolate the linear function exactly, and so
    do points next to it, where the routine extrapolates into the hole"""
    L = _lib()
    n = 13
    x = np.linspace(-1, 1, n)
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    lin = lambda a, b, c: 0.5 + 2 * a - b + 0.25 * c  # noqa: E731
    chr1 = _ball_mask(n, (6, 6, 6), 1.5)
    u1 = np.ascontiguousarray(lin(X, Y, Z).transpose(2, 1, 0)).reshape(-1)
    u1 = np.where(chr1 == EX, 1.0e6, u1)
    nf = 2 * n - 1
    u2 = np.zeros(nf ** 3)
    args = [n, n, n, nf, nf, nf, 1, 1, 1, 1, 1, 1, n, n, n, 1, 1, 1, 2, 2, 2, ord_]
    ex = C.c_double(EX)
    L.dminterp3d_(_dp(u1), _dp(u2), *[_ip(v) for v in args], _dp(chr1), C.byref(ex), _ip(1))
    xf = np.linspace(-1, 1, nf)
    Xf, Yf, Zf = np.meshgrid(xf, xf, xf, indexing="ij")
    want = lin(Xf, Yf, Zf)
    got = u2.reshape(nf, nf, nf).transpose(2, 1, 0)
    # fine points whose coarse cell (and, for cubic, its neighbours) is 2+ cells from the ball
    c = (np.arange(nf) / 2.0)
    Cx, Cy, Cz = np.meshgrid(c, c, c, indexing="ij")
    far = np.sqrt((Cx - 6) ** 2 + (Cy - 6) ** 2 + (Cz - 6) ** 2) > 1.5 + (2.0 if ord_ == 2 else 4.0)
    assert np.max(np.abs(got[far] - want[far])) < 1e-12
    assert np.isfinite(got).all()
