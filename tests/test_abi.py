"""The C-ABI library loads on a machine without a GPU and exports every
entry point include/pamr_gb300.h declares."""
import ctypes
import os
import re

from pamr_amrd_gb300 import build
from pamr_amrd_gb300.solver import lib

HDR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                   "pamr_gb300.h")


def declared():
    txt = open(HDR).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(pgb_\w+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    L = lib()
    names = declared()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_library_is_built_in_tree():
    path = build.build()
    assert os.path.dirname(path) == os.path.dirname(build.__file__)
    ctypes.CDLL(path)


def test_fortran_abi_dropin_exports_m_util_r8_symbols():
    """libpamr_gb300_f77.so carries the reference's m_util_r8.h entry points
    (Fortran ABI, trailing underscore) so an application relinks unchanged"""
    build.build()
    L = ctypes.CDLL(build.LIB_F77)
    for name in ("dmcopy3d_", "dmhwr3d_", "dmfwr3d_", "dminterp3d_", "dmdiss3d_", "linbnd3d_"):
        assert hasattr(L, name), name


def test_fortran_abi_half_weighting_refuses_unsupported_do_ex():
    """dmhwr3d masks its stencil legs for any nonzero do_ex but zeroes
    excised centres only for do_ex = 1 (src/m_util_r8.f:681-715); the
    drop-in implements 0 and 1 and leaves u2 unchanged for other values,
    before any device work (so this runs without a GPU)"""
    import numpy as np
    build.build()
    L = ctypes.CDLL(build.LIB_F77)
    u1 = np.arange(125, dtype=np.float64)
    u2 = np.full(27, -3.5)
    chr1 = np.zeros(125)
    ip = lambda v: ctypes.byref(ctypes.c_int(v))  # noqa: E731
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
    args = [dp(u1), dp(u2)] + [ip(v) for v in (5, 5, 5, 3, 3, 3, 1, 1, 1, 1, 1, 1, 3, 3, 3, 2, 2, 2, 1, 1, 1)]
    L.dmhwr3d_(*args, dp(chr1), ctypes.byref(ctypes.c_double(1.0)), ip(-1))
    assert np.all(u2 == -3.5)
