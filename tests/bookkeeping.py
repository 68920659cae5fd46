"""Expands libpamr_gb300's transfer plans into the m_util_r8 call sequence
the reference makes during solve_elliptics (build_mgh injections, then the
communications of each V-cycle in amrd/mg.c:84-201 order), so it can be
compared call for call with the op log of the compiled reference."""
from __future__ import annotations

import numpy as np

from pamr_amrd_gb300.solver import (PLAN_INJECT, PLAN_INJECT_INIT, PLAN_INTERP, PLAN_SYNC0,
                                    PLAN_SYNC1, Solver)

KIND_COPY, KIND_INTERP, KIND_HWR, KIND_FWR = 1, 2, 3, 4
F_SRC, F_U, F_RES = 0, 1, 2
F_SRC1 = 5   # sources 1..3 of an operator with several (library field order)


def _shape(s: Solver, L: int, idx: int):
    return s.box_info(L, idx)["shape"]


def _row(kind, src, dst, iv):
    r = np.zeros(34, dtype=np.int64)
    r[0] = kind
    r[4:7] = src
    r[7:10] = dst
    r[10:10 + len(iv)] = iv
    return r


def expand(s: Solver, which: int, L: int, gfn: dict, field: int | None = None):
    """m_util_r8 calls of one communication (src/transfer.c:946-1163)"""
    out = []
    for r in s.plan(which, L):
        Ls, si, Ld, di = r[0], r[1], r[2], r[3]
        n1, n2 = _shape(s, Ls, si), _shape(s, Ld, di)
        if which in (PLAN_SYNC0, PLAN_SYNC1, 2):
            g = gfn[field]
            iv = list(n1) + list(n2) + list(r[4:13]) + [1] * 6
            out.append(_row(KIND_COPY, (Ls, si, g), (Ld, di, g), iv))
        elif which in (PLAN_INJECT, PLAN_INJECT_INIT):
            irho = r[13]
            # local_transfer walks grid functions in PAMR gfn order (src/transfer.c:997)
            fields = sorted((f for f in range(8) if r[14 + f]), key=lambda f: gfn[f])
            for f in fields:
                op = r[14 + f]
                g = gfn[f]
                iv = list(n1) + list(n2) + list(r[4:13]) + [irho] * 3 + [1] * 3
                if op == 1:
                    out.append(_row(KIND_COPY, (Ls, si, g), (Ld, di, g), iv))
                else:
                    out.append(_row(KIND_HWR if op == 2 else KIND_FWR, (Ls, si, g), (Ld, di, g),
                                    iv + [0]))
        else:
            g = gfn[F_RES]
            irho, ordr = r[19], r[20]
            win = [(r[7] - 1) * irho + 1, (r[8] - 1) * irho + 1, (r[9] - 1) * irho + 1]
            if n1[2] == 1:
                win[2] = 1
            iv = list(n1) + win + list(r[4:7]) + [1, 1, 1] + list(r[7:10]) + [1, 1, 1] + \
                [irho] * 3 + [ordr, 0]
            out.append(_row(KIND_INTERP, (Ls, si, g), (-1, -1, -1), iv))
            iv2 = win + list(n2) + list(r[10:13]) + list(r[13:16]) + list(r[16:19]) + [1] * 6
            out.append(_row(KIND_COPY, (-1, -1, -1), (Ld, di, g), iv2))
    return out


def expected_calls(s: Solver, gfn: dict, ncycles: int, pre: int, pst: int):
    """build-time injections, then `ncycles` V-cycles (single-box coarsest levels)"""
    nl = s.num_levels()
    seq = []
    for L in range(nl - 1, 0, -1):
        seq += expand(s, PLAN_INJECT_INIT, L, gfn)
    for _ in range(ncycles):
        for L in range(nl, 0, -1):
            if L < nl:
                seq += expand(s, PLAN_SYNC0, L + 1, gfn, F_RES)
                seq += expand(s, PLAN_INJECT, L, gfn)
                seq += expand(s, PLAN_SYNC0, L, gfn, F_U)
            for it in range(pre):
                seq += expand(s, PLAN_SYNC1 if it else PLAN_SYNC0, L, gfn, F_U)
        for L in range(1, nl + 1):
            if L > 1:
                seq += expand(s, PLAN_INTERP, L, gfn)
            for it in range(pst):
                seq += expand(s, PLAN_SYNC1 if it else PLAN_SYNC0, L, gfn, F_U)
    return np.array(seq) if seq else np.zeros((0, 34), dtype=np.int64)


def reference_gfns(ref: dict) -> dict:
    g = ref["gfn"]
    out = {F_SRC: g["src"], F_U: g["u"], F_RES: g["res"]}
    for k in (1, 2, 3):
        if f"src{k}" in g:
            out[F_SRC1 + k - 1] = g[f"src{k}"]
    return out
