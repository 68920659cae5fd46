"""linbnd3d on the GPU (pgb_linbnd3d, and linbnd3d_ of the Fortran-ABI
drop-in library) against the oracle's restatement, bit for bit: every
which_bnd, random physical/AMR faces, with and without an excision mask,
on 3-D, 2-D and 1-D grids including extents small enough for later
statements to read what earlier ones wrote."""
import ctypes as C

import numpy as np
import pytest

from oracle import portrun

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
D = C.POINTER(C.c_double)


def _oracle(f, pb, which, shape, chr_, ex, do_ex):
    L = C.CDLL(portrun.build())
    L.oracle_linbnd3d.argtypes = [D, C.POINTER(C.c_int), C.c_int, C.c_int, C.c_int, C.c_int, D, C.c_double, C.c_int]
    f = f.copy()
    assert L.oracle_linbnd3d(f.ctypes.data_as(D), (C.c_int * 6)(*pb), which, *shape, chr_.ctypes.data_as(D), ex,
                             do_ex) == 0
    return f


@pytest.mark.parametrize("shape", [(40, 33, 29), (4, 5, 6), (3, 4, 3), (17, 13, 1), (9, 1, 1), (5, 3, 3)])
@pytest.mark.parametrize("which", [1, 2, 3])
@pytest.mark.parametrize("do_ex", [0, 1])
def test_linbnd3d_matches_oracle(shape, which, do_ex):
    from pamr_amrd_gb300.solver import lib
    rng = np.random.default_rng(sum(shape) * 10 + which * 2 + do_ex)
    n = int(np.prod(shape))
    f = rng.standard_normal(n)
    chr_ = np.where(rng.random(n) < 0.2, -1.0, 0.0)
    pb = [int(v) for v in rng.integers(0, 2, 6)]
    want = _oracle(f, pb, which, shape, chr_, -1.0, do_ex)
    L = lib()
    L.pgb_linbnd3d.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p,
                               C.c_double, C.c_int, C.c_void_p]
    df, dc = torch.from_numpy(f.copy()).cuda(), torch.from_numpy(chr_).cuda()
    rc = L.pgb_linbnd3d(df.data_ptr(), (C.c_int * 6)(*pb), which, *shape, dc.data_ptr(), -1.0, do_ex, None)
    torch.cuda.synchronize()
    assert rc == 0
    assert np.array_equal(df.cpu().numpy(), want)


def test_fortran_abi_linbnd3d_and_refusals():
    from pamr_amrd_gb300 import build
    from pamr_amrd_gb300.solver import lib
    shape = (12, 11, 10)
    rng = np.random.default_rng(3)
    f = rng.standard_normal(int(np.prod(shape)))
    chr_ = np.where(rng.random(f.size) < 0.2, -1.0, 0.0)
    pb = [1, 0, 1, 1, 0, 1]
    want = _oracle(f, pb, 3, shape, chr_, -1.0, 1)
    L = C.CDLL(build.LIB_F77)
    got = f.copy()
    ci = lambda v: C.byref(C.c_int(v))  # noqa: E731
    L.linbnd3d_(got.ctypes.data_as(D), (C.c_int * 6)(*pb), ci(3), ci(shape[0]), ci(shape[1]), ci(shape[2]),
                chr_.ctypes.data_as(D), C.byref(C.c_double(-1.0)), ci(1))
    assert np.array_equal(got, want)
    G = lib()
    G.pgb_linbnd3d.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p,
                               C.c_double, C.c_int, C.c_void_p]
    d = torch.zeros(100, dtype=torch.float64, device="cuda")
    assert G.pgb_linbnd3d(d.data_ptr(), (C.c_int * 6)(*pb), 3, 2, 5, 5, None, 0.0, 0, None) == 3
    assert G.pgb_linbnd3d(d.data_ptr(), (C.c_int * 6)(*pb), 4, 4, 5, 5, None, 0.0, 0, None) == 3
    assert G.pgb_linbnd3d(d.data_ptr(), (C.c_int * 6)(*pb), 3, 6, 1, 7, None, 0.0, 0, None) == 3
