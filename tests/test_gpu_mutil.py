"""The device m_util_r8 entry points (pgb_dmcopy3d, pgb_dmhwr3d,
pgb_dmfwr3d, pgb_dminterp3d) against the oracle's C restatement of
src/m_util_r8.f: bit-identical on random data, including strided copies,
offsets, 2-D/3-D and the out-of-range no-op."""
import ctypes as C

import numpy as np
import pytest

from oracle import portrun
from pamr_amrd_gb300.solver import lib

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _cpu():
    return C.CDLL(portrun.build())


def _ip(v):
    return C.byref(C.c_int(int(v)))


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _dev(a):
    return torch.from_numpy(a).cuda()


CASES = [
    # nx1 ny1 nz1 nx2 ny2 nz2 i1 j1 k1 i2 j2 k2 ni nj nk si1 sj1 sk1 si2 sj2 sk2
    (17, 17, 17, 9, 9, 9, 1, 1, 1, 1, 1, 1, 9, 9, 9, 2, 2, 2, 1, 1, 1),
    (33, 21, 1, 17, 11, 1, 3, 1, 1, 2, 1, 1, 14, 11, 1, 2, 2, 1, 1, 1, 1),
    (12, 10, 8, 12, 10, 8, 2, 3, 1, 1, 1, 2, 9, 6, 7, 1, 1, 1, 1, 1, 1),
    (9, 9, 9, 5, 5, 5, 1, 1, 1, 1, 1, 1, 6, 5, 5, 2, 2, 2, 1, 1, 1),    # out of range: no-op
]


@pytest.mark.parametrize("kind", ["dmcopy3d", "dmhwr3d", "dmfwr3d"])
@pytest.mark.parametrize("args", CASES)
def test_device_restriction_and_copy(kind, args):
    rng = np.random.default_rng(1)
    u1 = rng.standard_normal(args[0] * args[1] * args[2])
    u2 = rng.standard_normal(args[3] * args[4] * args[5])
    want = u2.copy()
    cpu = getattr(_cpu(), kind + "_")
    ex = C.c_double(0)
    if kind == "dmcopy3d":
        cpu(_dp(u1), _dp(want), *[_ip(v) for v in args])
    else:
        cpu(_dp(u1), _dp(want), *[_ip(v) for v in args], _dp(u1), C.byref(ex), _ip(0))
    d1, d2 = _dev(u1), _dev(u2)
    rc = getattr(lib(), "pgb_" + kind)(d1.data_ptr(), d2.data_ptr(), *args, None)
    torch.cuda.synchronize()
    assert rc == 0
    assert np.array_equal(d2.cpu().numpy(), want)


@pytest.mark.parametrize("ord_", [2, 4])
@pytest.mark.parametrize("geom", [(9, 9, 9, 9, 9, 9), (7, 5, 1, 7, 5, 1), (11, 6, 4, 6, 6, 4)])
def test_device_interp_window(ord_, geom):
    nx1, ny1, nz1, ni, nj, nk = geom
    rng = np.random.default_rng(2)
    u1 = rng.standard_normal(nx1 * ny1 * nz1)
    n2 = [(ni - 1) * 2 + 1, (nj - 1) * 2 + 1, (nk - 1) * 2 + 1 if nk > 1 else 1]
    u2 = np.zeros(n2[0] * n2[1] * n2[2])
    want = u2.copy()
    args = [nx1, ny1, nz1, *n2, 1, 1, 1, 1, 1, 1, ni, nj, nk, 1, 1, 1, 2, 2, 2, ord_]
    ex = C.c_double(0)
    _cpu().dminterp3d_(_dp(u1), _dp(want), *[_ip(v) for v in args], _dp(u1), C.byref(ex), _ip(0))
    d1, d2 = _dev(u1), _dev(u2)
    rc = lib().pgb_dminterp3d(d1.data_ptr(), d2.data_ptr(), *args, None)
    torch.cuda.synchronize()
    assert rc == 0
    assert np.array_equal(d2.cpu().numpy(), want)


# ------------------------------------------------------ excision (do_ex=1) --
EX = 1.0


def _mask(rng, n, nblobs=3):
    """0/EX mask with a few excised balls (and a sprinkling of single points)"""
    nx, ny, nz = n
    X, Y, Z = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    m = np.zeros((nx, ny, nz))
    for _ in range(nblobs):
        c = [rng.uniform(0, nx), rng.uniform(0, ny), rng.uniform(0, nz)]
        r = rng.uniform(0.8, 0.25 * min(nx, ny, max(nz, 4)))
        m[(X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2 <= r * r] = EX
    m[rng.random(m.shape) < 0.02] = EX
    return np.ascontiguousarray(m.transpose(2, 1, 0)).reshape(-1)


EX_RESTRICT = [
    (17, 17, 17, 9, 9, 9, 1, 1, 1, 1, 1, 1, 9, 9, 9, 2, 2, 2, 1, 1, 1),
    (33, 21, 1, 17, 11, 1, 3, 1, 1, 2, 1, 1, 14, 11, 1, 2, 2, 1, 1, 1, 1),
    (21, 19, 15, 11, 10, 8, 1, 1, 1, 1, 1, 1, 11, 10, 8, 2, 2, 2, 1, 1, 1),
]


@pytest.mark.parametrize("kind", ["dmhwr3d", "dmfwr3d"])
@pytest.mark.parametrize("args", EX_RESTRICT)
def test_device_excised_restriction(kind, args):
    rng = np.random.default_rng(3)
    u1 = rng.standard_normal(args[0] * args[1] * args[2])
    chr1 = _mask(rng, args[0:3])
    u2 = rng.standard_normal(args[3] * args[4] * args[5])
    want = u2.copy()
    ex = C.c_double(EX)
    getattr(_cpu(), kind + "_")(_dp(u1), _dp(want), *[_ip(v) for v in args], _dp(chr1), C.byref(ex), _ip(1))
    d1, d2, dc = _dev(u1), _dev(u2), _dev(chr1)
    rc = getattr(lib(), "pgb_" + kind + "_ex")(d1.data_ptr(), d2.data_ptr(), *args, dc.data_ptr(), EX, None)
    torch.cuda.synchronize()
    assert rc == 0
    assert np.array_equal(d2.cpu().numpy(), want)


# coarse grid, window (i1,j1,k1, ni,nj,nk) and the fine start, chosen so that
# every mask index the routines read stays inside the coarse grid
EX_INTERP = [
    ((9, 9, 9), (1, 1, 1, 9, 9, 9), (1, 1, 1)),        # whole grid onto an aligned fine grid
    ((13, 11, 1), (1, 1, 1, 13, 11, 1), (1, 1, 1)),    # 2-D
    ((16, 15, 14), (5, 4, 5, 7, 8, 6), (9, 7, 9)),     # inner window, fine margin of 4 cells
]


@pytest.mark.parametrize("ord_", [2, 4])
@pytest.mark.parametrize("geom", EX_INTERP)
def test_device_excised_interp(ord_, geom):
    (nx1, ny1, nz1), (i1, j1, k1, ni, nj, nk), (i2, j2, k2) = geom
    rng = np.random.default_rng(4)
    u1 = rng.standard_normal(nx1 * ny1 * nz1)
    chr1 = _mask(rng, (nx1, ny1, nz1))
    n2 = [i2 - 1 + (ni - 1) * 2 + 1 + (i2 - 1), j2 - 1 + (nj - 1) * 2 + 1 + (j2 - 1),
          (k2 - 1 + (nk - 1) * 2 + 1 + (k2 - 1)) if nk > 1 else 1]
    u2 = rng.standard_normal(n2[0] * n2[1] * n2[2])
    want = u2.copy()
    args = [nx1, ny1, nz1, *n2, i1, j1, k1, i2, j2, k2, ni, nj, nk, 1, 1, 1, 2, 2, 2, ord_]
    ex = C.c_double(EX)
    _cpu().dminterp3d_(_dp(u1), _dp(want), *[_ip(v) for v in args], _dp(chr1), C.byref(ex), _ip(1))
    d1, d2, dc = _dev(u1), _dev(u2), _dev(chr1)
    rc = lib().pgb_dminterp3d_ex(d1.data_ptr(), d2.data_ptr(), *args, dc.data_ptr(), EX, None)
    torch.cuda.synchronize()
    assert rc == 0
    assert np.array_equal(d2.cpu().numpy(), want)


# ------------------------------------------- Fortran-ABI drop-in (host arrays) --
def _f77():
    from pamr_amrd_gb300 import build
    return C.CDLL(build.LIB_F77)


@pytest.mark.parametrize("do_ex", [0, 1])
def test_fortran_abi_dropin_matches_oracle(do_ex):
    """the drop-in's dmhwr3d_/dmfwr3d_/dminterp3d_/dmcopy3d_ on host arrays
    give the oracle's results bit for bit"""
    rng = np.random.default_rng(5)
    n1, n2 = 17, 9
    u1 = rng.standard_normal(n1 ** 3)
    chr1 = _mask(rng, (n1, n1, n1)) if do_ex else np.zeros(n1 ** 3)
    ex = C.c_double(EX)
    F, O = _f77(), _cpu()
    args = [n1, n1, n1, n2, n2, n2, 1, 1, 1, 1, 1, 1, n2, n2, n2, 2, 2, 2, 1, 1, 1]
    for fn in ("dmhwr3d_", "dmfwr3d_"):
        a = rng.standard_normal(n2 ** 3)
        b = a.copy()
        getattr(F, fn)(_dp(u1), _dp(a), *[_ip(v) for v in args], _dp(chr1), C.byref(ex), _ip(do_ex))
        getattr(O, fn)(_dp(u1), _dp(b), *[_ip(v) for v in args], _dp(chr1), C.byref(ex), _ip(do_ex))
        assert np.array_equal(a, b), fn
    a = rng.standard_normal(n2 ** 3)
    b = a.copy()
    F.dmcopy3d_(_dp(u1), _dp(a), *[_ip(v) for v in args])
    O.dmcopy3d_(_dp(u1), _dp(b), *[_ip(v) for v in args])
    assert np.array_equal(a, b)
    c1 = rng.standard_normal(n2 ** 3)
    cchr = _mask(rng, (n2, n2, n2)) if do_ex else np.zeros(n2 ** 3)
    iargs = [n2, n2, n2, n1, n1, n1, 1, 1, 1, 1, 1, 1, n2, n2, n2, 1, 1, 1, 2, 2, 2, 2]
    a = rng.standard_normal(n1 ** 3)
    b = a.copy()
    F.dminterp3d_(_dp(c1), _dp(a), *[_ip(v) for v in iargs], _dp(cchr), C.byref(ex), _ip(do_ex))
    O.dminterp3d_(_dp(c1), _dp(b), *[_ip(v) for v in iargs], _dp(cchr), C.byref(ex), _ip(do_ex))
    assert np.array_equal(a, b)
