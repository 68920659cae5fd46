"""Known-answer tests of the oracle's restatement of linbnd3d
(src/m_util_r8.f:1957-2252): linear data is a fixed point of every face,
edge and corner mean; quadratic data shows the face means; which_bnd and
phys_bdy select the faces; an excised neighbour blocks a face update; the
Fortran's corner condition (A .and. B) .or. (all .and. X) updates a corner
next to an excised point when only the physical faces are selected; the
extents the Fortran stops on are refused, and so is Ny = 1 with Nz > 1,
where the Fortran indexes outside f."""
import ctypes as C

import numpy as np
import pytest

from oracle import portrun

D = C.POINTER(C.c_double)


@pytest.fixture(scope="module")
def lib():
    L = C.CDLL(portrun.build())
    L.oracle_linbnd3d.argtypes = [D, C.POINTER(C.c_int), C.c_int, C.c_int, C.c_int, C.c_int, D, C.c_double, C.c_int]
    return L


def run(lib, f, shape, which, pb=(1,) * 6, chr_=None, ex=-1.0):
    f = np.array(f, dtype=np.float64, order="F")
    c = np.asfortranarray(chr_ if chr_ is not None else np.zeros(shape), dtype=np.float64)
    rc = lib.oracle_linbnd3d(f.ctypes.data_as(D), (C.c_int * 6)(*pb), which, *shape, c.ctypes.data_as(D), ex,
                             0 if chr_ is None else 1)
    return rc, f


def grid(shape):
    return np.meshgrid(*[np.arange(1.0, n + 1) for n in shape], indexing="ij")


def test_linear_data_is_fixed(lib):
    shape = (6, 7, 8)
    i, j, k = grid(shape)
    f = 3 * i - 2 * j + 5 * k + 1
    rc, out = run(lib, f, shape, 3)
    assert rc == 0 and np.array_equal(out, f)


def test_quadratic_face_means(lib):
    shape = (7, 6, 5)
    i, _, _ = grid(shape)
    rc, out = run(lib, i * i, shape, 3)
    assert rc == 0
    assert np.all(out[1, 2:4, 2:3] == 5.0)          # (1 + 9) / 2 at i = 2
    assert np.all(out[5, 2:4, 2:3] == 37.0)         # (25 + 49) / 2 at i = 6
    assert np.all(out[2:5, 2:4, 2:3] == (i * i)[2:5, 2:4, 2:3])


def test_only_selected_faces_change(lib):
    shape = (6, 6, 6)
    i, j, k = grid(shape)
    f = i * i + j * j + k * k
    rc, out = run(lib, f, shape, 1, pb=(1, 0, 0, 0, 0, 0))
    changed = out != f
    assert rc == 0 and changed[1].any() and not changed[2:].any() and not changed[0].any()
    rc, out2 = run(lib, f, shape, 2, pb=(1, 0, 0, 0, 0, 0))   # AMR faces: every face but x-lower
    assert not (out2 != f)[1, 2:4, 2:4].any() and (out2 != f)[4].any()


def test_excised_neighbour_blocks_the_face(lib):
    shape = (6, 6, 6)
    i, _, _ = grid(shape)
    f = i * i
    chr_ = np.zeros(shape)
    chr_[2, 3, 3] = -1.0                             # point (3, 4, 4) excised
    rc, out = run(lib, f, shape, 3, chr_=chr_)
    assert out[1, 3, 3] == 4.0 and out[1, 2, 2] == 5.0


def test_corner_condition_precedence(lib):
    shape = (6, 6, 6)
    i, j, k = grid(shape)
    f = i * j * k
    chr_ = np.zeros(shape)
    chr_[0, 0, 0] = -1.0                             # (1, 1, 1) excised
    rc, out = run(lib, f, shape, 1, pb=(1,) * 6, chr_=chr_)
    want = 0.125 * (27 + 9 + 9 + 9 + 3 + 3 + 3 + 1)  # physical faces only: (A and B) holds, X not tested
    assert out[1, 1, 1] == want
    rc, out = run(lib, f, shape, 3, pb=(1,) * 6, chr_=chr_)
    assert out[1, 1, 1] == 8.0                        # all faces: X is tested, corner kept


@pytest.mark.parametrize("shape", [(2, 5, 5), (5, 2, 5), (5, 5, 2), (6, 1, 7)])
def test_invalid_extents(lib, shape):
    assert run(lib, np.zeros(shape), shape, 3)[0] == 1
