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
