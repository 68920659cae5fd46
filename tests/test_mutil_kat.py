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
