"""Python front end of libpamr_gb300 (ctypes over the C ABI in
include/pamr_gb300.h).

This is the interface the tests and the benchmark call; a C application
calls the same entry points directly. There is no CPU fallback: if the
library or a GPU is missing, calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build
from .workloads import Case

_lib = None

PLAN_SYNC0, PLAN_SYNC1, PLAN_SYNC_COARSEST, PLAN_INJECT, PLAN_INJECT_INIT, PLAN_INTERP = range(6)


class PgbError(RuntimeError):
    pass


class MGParams(C.Structure):
    _fields_ = [("pre_swp", C.c_int), ("pst_swp", C.c_int), ("max_iter", C.c_int),
                ("min_iter", C.c_int), ("max_citer", C.c_int), ("tol", C.c_double),
                ("crtol", C.c_double), ("w0_r", C.c_double), ("w0_i", C.c_double),
                ("min_cwidth", C.c_int), ("restr_u", C.c_int), ("restr_res", C.c_int),
                ("restr_src", C.c_int), ("interp_order", C.c_int), ("interp_buffer", C.c_int),
                ("precision", C.c_int)]


class CreateArgs(C.Structure):
    _fields_ = [("dim", C.c_int), ("op", C.c_void_p), ("base_shape", C.c_int * 3),
                ("base_bbox", C.c_double * 6), ("ngrids", C.c_int),
                ("grid_level", C.POINTER(C.c_int)), ("grid_bbox", C.POINTER(C.c_double)),
                ("params", MGParams), ("min_level", C.c_int), ("restr_src", C.c_int * 4),
                ("flags", C.c_int), ("nvar", C.c_int), ("var_op", C.c_void_p * 4)]


def lib(build: bool = True):
    """Loads libpamr_gb300.so (building it first if needed)."""
    global _lib
    if _lib is None:
        path = _build.build() if build else _build.LIB
        if not os.path.exists(path):
            raise PgbError(f"{path} missing: run pamr_amrd_gb300.build.build()")
        L = C.CDLL(path)
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int)
        vp = C.c_void_p
        L.pgb_last_error.restype = C.c_char_p
        L.pgb_create.argtypes = [C.c_int, C.c_int, ip, dp, C.c_int, ip, dp, C.POINTER(MGParams),
                                 C.c_int, C.POINTER(vp)]
        L.pgb_create_ex.argtypes = [C.POINTER(CreateArgs), C.POINTER(vp)]
        L.pgb_default_create_args.argtypes = [C.POINTER(CreateArgs)]
        L.pgb_operator_create.argtypes = [C.c_int, C.c_char_p, C.c_char_p, C.POINTER(vp)]
        L.pgb_operator_builtin.argtypes = [C.c_int, C.POINTER(vp)]
        L.pgb_operator_destroy.argtypes = [vp]
        L.pgb_operator_kind.argtypes = [vp]
        L.pgb_operator_nsrc.argtypes = [vp]
        L.pgb_operator_eval.argtypes = [vp, C.c_double, C.c_double, C.c_double, dp, dp, dp]
        L.pgb_set_source.argtypes = [vp, C.c_int, C.c_int, dp]
        L.pgb_set_source_device.argtypes = [vp, C.c_int, C.c_int, vp]
        L.pgb_destroy.argtypes = [vp]
        L.pgb_grid_shape.argtypes = [vp, C.c_int, ip]
        L.pgb_set_grid.argtypes = [vp, C.c_int, dp, dp]
        L.pgb_get_grid.argtypes = [vp, C.c_int, dp]
        L.pgb_set_grid_device.argtypes = [vp, C.c_int, vp, vp]
        L.pgb_get_grid_device.argtypes = [vp, C.c_int, vp]
        L.pgb_solve.argtypes = [vp, ip, dp, dp, C.c_int]
        L.pgb_prepare.argtypes = [vp]
        L.pgb_vcycle.argtypes = [vp, dp]
        L.pgb_stream.argtypes = [vp]
        L.pgb_stream.restype = vp
        L.pgb_stats.argtypes = [vp, ip, C.POINTER(C.c_long), dp]
        L.pgb_trace_enable.argtypes = [vp, C.c_int]
        L.pgb_trace_fetch.argtypes = [vp, ip, ip, ip, ip, dp, C.c_int, ip]
        L.pgb_num_levels.argtypes = [vp]
        L.pgb_level_nbox.argtypes = [vp, C.c_int]
        L.pgb_box_info.argtypes = [vp, C.c_int, C.c_int, ip, dp, ip, ip]
        L.pgb_box_cmask.argtypes = [vp, C.c_int, C.c_int, C.c_int, dp]
        L.pgb_plan_dump.argtypes = [vp, C.c_int, C.c_int, ip, C.c_int]
        L.pgb_default_params.argtypes = [C.POINTER(MGParams)]
        L.pgb_launch_count.restype = C.c_longlong
        L.pgb_time_relax.argtypes = [vp, C.c_int, C.c_int, dp, dp]
        L.pgb_level_tuning.argtypes = [vp, C.c_int, ip, ip]
        L.pgb_tail_levels.argtypes = [vp, ip]
        for name in ("pgb_dmcopy3d", "pgb_dmhwr3d", "pgb_dmfwr3d"):
            getattr(L, name).argtypes = [vp, vp] + [C.c_int] * 21 + [vp]
        L.pgb_dminterp3d.argtypes = [vp, vp] + [C.c_int] * 22 + [vp]
        for name in ("pgb_dmhwr3d_ex", "pgb_dmfwr3d_ex"):
            getattr(L, name).argtypes = [vp, vp] + [C.c_int] * 21 + [vp, C.c_double, vp]
        L.pgb_dminterp3d_ex.argtypes = [vp, vp] + [C.c_int] * 22 + [vp, C.c_double, vp]
        _lib = L
    return _lib


def launch_count() -> int:
    return int(lib().pgb_launch_count())


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _check(rc: int):
    if rc != 0:
        raise PgbError(f"libpamr_gb300 error {rc}: {lib().pgb_last_error().decode()}")


def params_from(case: Case) -> MGParams:
    p = case.params
    m = MGParams()
    lib().pgb_default_params(C.byref(m))
    m.pre_swp, m.pst_swp, m.max_iter, m.min_iter = p.pre_swp, p.pst_swp, p.max_iter, p.min_iter
    m.max_citer, m.tol, m.crtol, m.w0_r, m.w0_i = p.max_citer, p.tol, p.crtol, p.w0_r, p.w0_i
    m.min_cwidth, m.restr_u, m.restr_res, m.restr_src = (p.min_cwidth, p.restr_u, p.restr_res,
                                                         p.restr_src)
    m.interp_order, m.interp_buffer = p.interp_order, 2
    m.precision = getattr(p, "precision", 0)
    return m


class Operator:
    """A level operator: a built-in PDE kind, or the expressions an
    application registers (pgb_operator_create)."""

    def __init__(self, pde: int = None, nsrc: int = 1, lop: str = None, jac: str = None):
        L = lib()
        h = C.c_void_p()
        if lop is None:
            _check(L.pgb_operator_builtin(pde, C.byref(h)))
        else:
            _check(L.pgb_operator_create(nsrc, lop.encode(), jac.encode(), C.byref(h)))
        self.h = h

    @classmethod
    def for_case(cls, case: Case, var: int = 0) -> "Operator":
        """the operator of elliptic variable `var` of the case"""
        from .workloads import OPERATORS, VAR_OPERATORS
        if case.pde in VAR_OPERATORS:
            n, pairs = VAR_OPERATORS[case.pde]
            return cls(nsrc=n, lop=pairs[var][0], jac=pairs[var][1])
        if case.pde in OPERATORS:
            n, lop, jac = OPERATORS[case.pde]
            return cls(nsrc=n, lop=lop, jac=jac)
        return cls(pde=case.pde)

    def kind(self) -> int:
        return lib().pgb_operator_kind(self.h)

    def close(self):
        if self.h:
            lib().pgb_operator_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Solver:
    """One AMR hierarchy on the GPU (or, with host_only, just its plans)."""

    def __init__(self, case: Case, host_only: bool = False, op: Operator = None):
        L = lib()
        self.case = case
        n = len(case.grids)
        self._lev = (C.c_int * n)(*[g.level for g in case.grids])
        bb = np.zeros((n, 6))
        for i, g in enumerate(case.grids):
            bb[i, :len(g.bbox)] = g.bbox
        self._bb = np.ascontiguousarray(bb)
        op = op or Operator.for_case(case)
        a = CreateArgs()
        L.pgb_default_create_args(C.byref(a))
        a.dim = case.dim
        a.op = op.h
        for d in range(3):
            a.base_shape[d] = case.base_shape[d]
        for d, v in enumerate(list(case.base_bbox) + [0.0] * (6 - len(case.base_bbox))):
            a.base_bbox[d] = v
        a.ngrids = n
        a.grid_level = self._lev
        a.grid_bbox = _dp(self._bb)
        a.params = params_from(case)
        a.min_level = case.min_level
        for k in range(1, case.nsrc):
            a.restr_src[k] = case.restr_src_k(k)
        a.flags = 1 if host_only else 0
        a.nvar = case.nvar
        self._var_ops = [Operator.for_case(case, v) for v in range(1, case.nvar)]
        for v, o in enumerate(self._var_ops, start=1):
            a.var_op[v] = o.h
        h = C.c_void_p()
        _check(L.pgb_create_ex(C.byref(a), C.byref(h)))
        self.h = h
        self.host_only = host_only
        self.op_kind = op.kind()

    def close(self):
        if self.h:
            lib().pgb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------- data --
    def _in_hierarchy(self, i: int) -> bool:
        return self.case.grids[i].level >= self.case.min_level

    def set_inputs(self, u=None, src=None):
        u = u if u is not None else self.case.u0
        src = src if src is not None else self.case.src
        for i, (a, s) in enumerate(zip(u, src)):
            if not self._in_hierarchy(i):
                continue
            a = np.ascontiguousarray(a, dtype=np.float64)
            s = np.ascontiguousarray(s, dtype=np.float64)
            _check(lib().pgb_set_grid(self.h, i, _dp(a), _dp(s)))
            for k in range(1, self.case.nsrc):
                sk = np.ascontiguousarray(self.case.source(k)[i], dtype=np.float64)
                _check(lib().pgb_set_source(self.h, i, k, _dp(sk)))
            for v in range(1, self.case.nvar):
                uv = np.ascontiguousarray(self.case.var(v)[i], dtype=np.float64)
                _check(lib().pgb_set_var(self.h, i, v, _dp(uv)))

    def get_u(self):
        out = []
        for g in self.case.grids:
            a = np.empty(g.size)
            out.append(a)
        for i, a in enumerate(out):
            if self._in_hierarchy(i):
                _check(lib().pgb_get_grid(self.h, i, _dp(a)))
            else:   # outside the MG hierarchy: unchanged by a solve
                a[:] = self.case.u0[i]
        return out

    def get_sources(self):
        """every source of every input grid in the hierarchy (None for grids
        below it): out[k][i] = source k of grid i"""
        out = [[None] * len(self.case.grids) for _ in range(self.case.nsrc)]
        for L in range(1, self.num_levels() + 1):
            for idx in range(self.level_nbox(L)):
                info = self.box_info(L, idx)
                g = info["amr_grid"]
                if g < 0 or out[0][g] is not None:
                    continue
                for k in range(self.case.nsrc):
                    a = np.empty(self.case.grids[g].size)
                    _check(lib().pgb_box_get(self.h, L, idx, 4 + k, _dp(a)))
                    out[k][g] = a
        return out

    def get_vars(self):
        """every elliptic variable on every input grid: out[v][i]"""
        out = [self.get_u()]
        for v in range(1, self.case.nvar):
            vals = []
            for i, g in enumerate(self.case.grids):
                a = np.empty(g.size)
                if self._in_hierarchy(i):
                    _check(lib().pgb_get_var(self.h, i, v, _dp(a)))
                else:
                    a[:] = self.case.var(v)[i]
                vals.append(a)
            out.append(vals)
        return out

    # ------------------------------------------------------------ solve --
    def solve(self):
        cap = max(1, self.case.params.max_iter)
        res = np.zeros(cap)
        it = C.c_int()
        rf = C.c_double()
        _check(lib().pgb_solve(self.h, C.byref(it), C.byref(rf), _dp(res), cap))
        return {"iters": it.value, "res": res[:it.value].copy(), "res_final": rf.value}

    def prepare(self):
        _check(lib().pgb_prepare(self.h))

    def vcycle(self) -> float:
        r = C.c_double()
        _check(lib().pgb_vcycle(self.h, C.byref(r)))
        return r.value

    def stats(self):
        v, c, ms = C.c_int(), C.c_long(), C.c_double()
        lib().pgb_stats(self.h, C.byref(v), C.byref(c), C.byref(ms))
        return {"vcycles": v.value, "coarsest_iters": c.value, "device_ms": ms.value}

    def level_tuning(self, L: int):
        """(tile planes, FP32 sweeps per launch) the autotuner chose for level L"""
        tz, f = C.c_int(), C.c_int()
        _check(lib().pgb_level_tuning(self.h, L, C.byref(tz), C.byref(f)))
        return tz.value, f.value

    def tail_levels(self):
        """(MG levels 1..n run by the small-level kernel, its cluster's CTAs);
        (0, 0) when every pass is a launch of its own"""
        n = C.c_int()
        lv = lib().pgb_tail_levels(self.h, C.byref(n))
        return lv, n.value

    def time_relax(self, L: int, reps: int = 20):
        ms, by = C.c_double(), C.c_double()
        _check(lib().pgb_time_relax(self.h, L, reps, C.byref(ms), C.byref(by)))
        return ms.value, by.value

    def amr_interp(self, lc: int, amr_bdy_width: int = 0, order: int = 2):
        """PAMR_interp (width 0) / PAMR_AMR_bdy_interp of u from AMR level lc to lc+1"""
        _check(lib().pgb_amr_interp(self.h, lc, amr_bdy_width, order))

    def regrid_from(self, old: "Solver", order: int = 2, min_level: int = 2):
        """u and the sources of this solver's AMR levels from ``old``, the
        solver of the hierarchy before the regrid (pgb_regrid: PAMR's
        init_new_cgh transfers, interpolation from level L-1 on levels >=
        min_level, then copies from level L)"""
        L = lib()
        L.pgb_regrid.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int]
        _check(L.pgb_regrid(self.h, old.h, order, min_level))

    def checkpoint_save(self, path: str):
        L = lib()
        L.pgb_checkpoint_save.argtypes = [C.c_void_p, C.c_char_p]
        _check(L.pgb_checkpoint_save(self.h, path.encode()))

    def checkpoint_load(self, path: str):
        L = lib()
        L.pgb_checkpoint_load.argtypes = [C.c_void_p, C.c_char_p]
        _check(L.pgb_checkpoint_load(self.h, path.encode()))

    def set_inputs_device(self, u_ptrs, src_ptrs, extra_src_ptrs=()):
        """device pointers per grid: u, source 0, and (extra_src_ptrs[k-1][i])
        source k"""
        for i, (a, b) in enumerate(zip(u_ptrs, src_ptrs)):
            if not self._in_hierarchy(i):
                continue
            _check(lib().pgb_set_grid_device(self.h, i, a, b))
            for k, ptrs in enumerate(extra_src_ptrs, start=1):
                _check(lib().pgb_set_source_device(self.h, i, k, ptrs[i]))

    def stream(self) -> int:
        return lib().pgb_stream(self.h)

    def trace_enable(self, cap: int):
        _check(lib().pgb_trace_enable(self.h, cap))
        self._trace_cap = cap

    def trace_fetch(self):
        cap = self._trace_cap
        k, l, b, r = (np.zeros(cap, dtype=np.int32) for _ in range(4))
        nrm = np.zeros(cap)
        n = C.c_int()
        ip = C.POINTER(C.c_int)
        _check(lib().pgb_trace_fetch(self.h, k.ctypes.data_as(ip), l.ctypes.data_as(ip),
                                     b.ctypes.data_as(ip), r.ctypes.data_as(ip), _dp(nrm), cap,
                                     C.byref(n)))
        m = n.value
        return {"kind": k[:m], "L": l[:m], "idx": b[:m], "repeat": r[:m], "norm": nrm[:m]}

    # ---------------------------------------------------------- queries --
    def num_levels(self) -> int:
        return lib().pgb_num_levels(self.h)

    def level_nbox(self, L: int) -> int:
        return lib().pgb_level_nbox(self.h, L)

    def box_info(self, L: int, idx: int):
        shape = (C.c_int * 3)()
        bb = (C.c_double * 6)()
        co, ag = C.c_int(), C.c_int()
        _check(lib().pgb_box_info(self.h, L, idx, shape, bb, C.byref(co), C.byref(ag)))
        return {"shape": tuple(shape), "bbox": tuple(bb), "coarsest": co.value,
                "amr_grid": ag.value}

    def cmask(self, L: int, idx: int, kind: str) -> np.ndarray:
        sh = self.box_info(L, idx)["shape"]
        out = np.zeros(sh[0] * sh[1] * sh[2])
        _check(lib().pgb_box_cmask(self.h, L, idx, 1 if kind == "child" else 0, _dp(out)))
        return out

    def plan(self, which: int, L: int) -> np.ndarray:
        n = lib().pgb_plan_dump(self.h, which, L, None, 0)
        if n < 0:
            _check(-n)
        rows = np.zeros((max(n, 1), 24), dtype=np.int32)
        lib().pgb_plan_dump(self.h, which, L, rows.ctypes.data_as(C.POINTER(C.c_int)), n)
        return rows[:n]
