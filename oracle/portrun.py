"""ctypes front end of the oracle port (oracle/port/mg_port.c).

TEST INFRASTRUCTURE (oracle only): used by tests/, __graft_entry__.smoke()
and bench.py's CPU-baseline arm. ``build()`` compiles the port with gcc
(-ffp-contract=off so x86 and Arm round identically).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "port", "libmgport.so")
# the same sources built for the timed CPU baseline: -O3 and the host's own
# instruction set (-ffp-contract=off keeps the arithmetic; the parity checker
# uses LIB, built without machine-specific flags so that x86 and Arm agree)
LIB_FAST = os.path.join(HERE, "port", "libmgport_fast.so")
SOURCES = [os.path.join(HERE, "port", "mg_port.c"), os.path.join(HERE, "mg_ops.c"),
           os.path.join(HERE, "m_util_r8.c"), os.path.join(HERE, "bo_ops.c")]


def build(force: bool = False, fast: bool = False) -> str:
    lib = LIB_FAST if fast else LIB
    newest = max(os.path.getmtime(s) for s in SOURCES)
    if force or not os.path.exists(lib) or os.path.getmtime(lib) < newest:
        opt = ["-O3", "-march=native"] if fast else ["-O2"]
        cmd = ["gcc"] + opt + ["-ffp-contract=off", "-fno-fast-math", "-std=gnu11", "-fPIC",
                               "-shared", "-o", lib] + SOURCES + ["-lm"]
        subprocess.run(cmd, check=True)
    return lib


class _Case(C.Structure):
    _fields_ = [("dim", C.c_int), ("pde", C.c_int), ("ngrids", C.c_int),
                ("base_shape", C.c_int * 3), ("base_bbox", C.c_double * 6),
                ("lev", C.POINTER(C.c_int)), ("bbox", C.POINTER(C.c_double)),
                ("u", C.POINTER(C.POINTER(C.c_double))),
                ("src", C.POINTER(C.POINTER(C.c_double))),
                ("pre_swp", C.c_int), ("pst_swp", C.c_int), ("max_iter", C.c_int),
                ("min_iter", C.c_int), ("max_citer", C.c_int),
                ("tol", C.c_double), ("crtol", C.c_double), ("w0_r", C.c_double),
                ("w0_i", C.c_double), ("min_cwidth", C.c_int),
                ("restr_u", C.c_int), ("restr_res", C.c_int), ("restr_src", C.c_int),
                ("interp_order", C.c_int), ("interp_buffer", C.c_int),
                ("srcx", C.POINTER(C.POINTER(C.c_double)) * 3), ("restr_srcx", C.c_int * 3),
                ("min_level", C.c_int)]


class _Result(C.Structure):
    _fields_ = [("iters", C.c_int), ("n_levels", C.c_int), ("res", C.POINTER(C.c_double)),
                ("hk_cap", C.c_int), ("hk_n", C.c_int),
                ("hk_kind", C.POINTER(C.c_int)), ("hk_L", C.POINTER(C.c_int)),
                ("hk_idx", C.POINTER(C.c_int)), ("hk_norm", C.POINTER(C.c_double))]


_libs = {}


def _load(fast: bool = False):
    if fast not in _libs:
        L = C.CDLL(build(fast=fast))
        L.port_solve.argtypes = [C.POINTER(_Case), C.POINTER(_Result)]
        L.port_solve.restype = C.c_int
        _libs[fast] = L
    return _libs[fast]


def solve(case, hook_cap: int = 0, fast: bool = False) -> dict:
    """Solves ``case`` with the oracle port. Returns the solution per input
    grid, the V-cycle count, per-cycle finest residuals and (if hook_cap>0)
    the hook log (kind 0 relax, 1 residual, 2 lop; level; grid index; norm)."""
    lib = _load(fast)
    n = len(case.grids)
    p = case.params
    lev = (C.c_int * n)(*[g.level for g in case.grids])
    bb = np.zeros((n, 6))
    for i, g in enumerate(case.grids):
        bb[i, :len(g.bbox)] = g.bbox
    bb = np.ascontiguousarray(bb)
    u = [np.array(a, dtype=np.float64, copy=True) for a in case.u0]
    s = [np.ascontiguousarray(a, dtype=np.float64) for a in case.src]
    up = (C.POINTER(C.c_double) * n)(*[a.ctypes.data_as(C.POINTER(C.c_double)) for a in u])
    sp = (C.POINTER(C.c_double) * n)(*[a.ctypes.data_as(C.POINTER(C.c_double)) for a in s])
    c = _Case()
    c.dim, c.pde, c.ngrids = case.dim, case.pde, n
    for d in range(3):
        c.base_shape[d] = case.base_shape[d]
    for k in range(2 * case.dim):
        c.base_bbox[k] = case.base_bbox[k]
    c.lev = lev
    c.bbox = bb.ctypes.data_as(C.POINTER(C.c_double))
    c.u, c.src = up, sp
    c.pre_swp, c.pst_swp, c.max_iter = p.pre_swp, p.pst_swp, p.max_iter
    c.min_iter, c.max_citer = p.min_iter, p.max_citer
    c.tol, c.crtol, c.w0_r, c.w0_i = p.tol, p.crtol, p.w0_r, p.w0_i
    c.min_cwidth = p.min_cwidth
    c.restr_u, c.restr_res, c.restr_src = p.restr_u, p.restr_res, p.restr_src
    c.interp_order, c.interp_buffer = p.interp_order, 2
    keep = []
    for k in range(1, case.nsrc):
        sk = [np.ascontiguousarray(a, dtype=np.float64) for a in case.source(k)]
        arr = (C.POINTER(C.c_double) * n)(*[a.ctypes.data_as(C.POINTER(C.c_double)) for a in sk])
        keep.append((sk, arr))
        c.srcx[k - 1] = C.cast(arr, C.POINTER(C.POINTER(C.c_double)))
        c.restr_srcx[k - 1] = case.restr_src_k(k)
    c.min_level = case.min_level
    res = np.zeros(max(1, p.max_iter))
    r = _Result()
    r.res = res.ctypes.data_as(C.POINTER(C.c_double))
    hk = {k: np.zeros(max(1, hook_cap), dtype=np.int32) for k in ("kind", "L", "idx")}
    hkn = np.zeros(max(1, hook_cap))
    r.hk_cap = hook_cap
    r.hk_kind = hk["kind"].ctypes.data_as(C.POINTER(C.c_int))
    r.hk_L = hk["L"].ctypes.data_as(C.POINTER(C.c_int))
    r.hk_idx = hk["idx"].ctypes.data_as(C.POINTER(C.c_int))
    r.hk_norm = hkn.ctypes.data_as(C.POINTER(C.c_double))
    rc = lib.port_solve(C.byref(c), C.byref(r))
    if rc:
        raise RuntimeError(f"port_solve failed ({rc})")
    out = {"iters": r.iters, "n_levels": r.n_levels, "res": res[:r.iters].copy(), "u": u}
    if hook_cap:
        m = r.hk_n
        out["hooks"] = {"kind": hk["kind"][:m].copy(), "L": hk["L"][:m].copy(),
                        "idx": hk["idx"][:m].copy(), "norm": hkn[:m].copy()}
    return out
