"""Berger-Oliger bookkeeping of the elliptic variables on the device
(binding of pgb_mg_extrap, pgb_update_mg_extrap_vars, pgb_set_mg_brs_vars
in libpamr_gb300; the reference's loops are amrd/evolve.c:344-366,
1640-1700, 1621-1638). Grids are lists of device pointers (ints) with
their levels and point counts."""
from __future__ import annotations

import ctypes as C

from .solver import _check, lib

ETM1, TN = 0, 1   # AMRD_MG_EXTRAP_2ND_FROM_ETM1, AMRD_MG_EXTRAP_2ND_FROM_TN
_bound = False


def _lib():
    global _bound
    L = lib()
    if not _bound:
        vp, pp = C.c_void_p, C.POINTER(C.c_void_p)
        L.pgb_mg_extrap.argtypes = [C.c_int] + [C.c_double] * 4 + [vp] * 4 + [C.c_long, vp]
        L.pgb_update_mg_extrap_vars.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int), C.c_int,
                                                C.POINTER(C.c_int), pp, pp, pp, pp, C.POINTER(C.c_long),
                                                C.c_double, vp]
        L.pgb_set_mg_brs_vars.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), pp, pp,
                                          C.POINTER(C.c_long), vp]
        _bound = True
    return L


def _ptrs(a):
    return (C.c_void_p * len(a))(*a)


def mg_extrap(method, tnp1, tnp1_lm1, dt, dt_lm1, mgf0, mgf1, etm1, etm2, n, stream=None):
    _check(_lib().pgb_mg_extrap(method, tnp1, tnp1_lm1, dt, dt_lm1, mgf0, mgf1, etm1, etm2, n, stream))


def update_mg_extrap_vars(L1, Lf, rho_tm, level, etm1, etm2, mgf1, brs, n, eps_c=1.0, stream=None):
    g = len(level)
    rho = (C.c_int * len(rho_tm))(*rho_tm)
    _check(_lib().pgb_update_mg_extrap_vars(L1, Lf, rho, g, (C.c_int * g)(*level), _ptrs(etm1), _ptrs(etm2),
                                            _ptrs(mgf1), _ptrs(brs), (C.c_long * g)(*n), eps_c, stream))


def set_mg_brs_vars(L1, L2, level, brs, mgf1, n, stream=None):
    g = len(level)
    _check(_lib().pgb_set_mg_brs_vars(L1, L2, g, (C.c_int * g)(*level), _ptrs(brs), _ptrs(mgf1),
                                      (C.c_long * g)(*n), stream))
