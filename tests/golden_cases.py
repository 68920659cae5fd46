"""Loads the golden fixtures of tests/golden/ (made by make_golden.py from
the compiled reference) back into workload Cases plus the reference's
recorded outputs."""
from __future__ import annotations

import glob
import os

import numpy as np

from pamr_amrd_gb300 import workloads as W

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def files():
    """the solve fixtures"""
    return sorted(f for f in glob.glob(os.path.join(GOLDEN, "*.npz"))
                  if not os.path.basename(f).startswith(("amr_interp_", "dropin_", "regrid", "coupled_")))


def dropin_files():
    """the drop-in application fixtures"""
    return sorted(glob.glob(os.path.join(GOLDEN, "dropin_*.npz")))


def load_dropin(path: str):
    """(case, mode, arg, level, what the reference build of the application
    wrote: iters, residuals, and u / cmask per AMR grid in PAMR order)"""
    z = np.load(path)
    dim = int(z["dim"])
    grids = []
    for row in z["grids"]:
        lev, s0, s1, s2 = (int(v) for v in row[:4])
        grids.append(W.Grid(lev, tuple(float(v) for v in row[4:4 + 2 * dim]), (s0, s1, s2)))
    ip = [int(v) for v in z["params"]]
    fp = [float(v) for v in z["fparams"]]
    params = W.MGParams(pre_swp=ip[0], pst_swp=ip[1], max_iter=ip[2], min_iter=ip[3],
                        max_citer=ip[4], min_cwidth=ip[5], restr_u=ip[6], restr_res=ip[7],
                        restr_src=ip[8], interp_order=ip[9], tol=fp[0], crtol=fp[1],
                        w0_r=fp[2], w0_i=fp[3])
    offs = np.cumsum([0] + [g.size for g in grids])
    split = lambda a: [a[offs[i]:offs[i + 1]].copy() for i in range(len(grids))]  # noqa: E731
    case = W.Case(str(z["name"]), int(z["pde"]), dim, tuple(int(v) for v in z["base_shape"]),
                  tuple(float(v) for v in z["base_bbox"]), grids, split(z["u0"]), split(z["src"]), params,
                  src_extra=[split(z["src1"])])
    if "u1_0" in z.files and len(z["u1_0"]):   # a coupled case's second variable
        case.u_extra = [split(z["u1_0"])]
    og, out = z["out_grids"], []
    off = 0
    for row in og:
        n = int(row[1] * row[2] * row[3])
        out.append({"level": int(row[0]), "shape": tuple(int(v) for v in row[1:4]),
                    "bbox": tuple(float(v) for v in row[4:10]), "u": z["out_u"][off:off + n].copy(),
                    "cmask": z["out_cmask"][off:off + n].astype(np.float64)})
        if "out_w" in z.files and len(z["out_w"]):
            out[-1]["w"] = z["out_w"][off:off + n].copy()
        off += n
    ref = {"iters": int(z["iters"]), "res": z["res"].copy(), "grids": out}
    return case, int(z["mode"]), int(z["arg"]), int(z["level"]), ref


def interp_files():
    """the AMR-hierarchy interpolation fixtures"""
    return sorted(glob.glob(os.path.join(GOLDEN, "amr_interp_*.npz")))


def load_interp(path: str):
    """(case with the fixture's seeded random u and zero source, (lc, width,
    order), u the reference's PAMR_interp / PAMR_AMR_bdy_interp left on every
    grid)"""
    z = np.load(path)
    dim = int(z["dim"])
    grids = []
    for row in z["grids"]:
        lev, s0, s1, s2 = (int(v) for v in row[:4])
        grids.append(W.Grid(lev, tuple(float(v) for v in row[4:4 + 2 * dim]), (s0, s1, s2)))
    rng = np.random.default_rng(int(z["seed"]))
    u0 = [rng.standard_normal(g.size) for g in grids]
    case = W.Case(str(z["name"]), int(z["pde"]), dim, tuple(int(v) for v in z["base_shape"]),
                  tuple(float(v) for v in z["base_bbox"]), grids, u0, [np.zeros(g.size) for g in grids],
                  W.MGParams(min_cwidth=9 if int(z["pde"]) == W.CONFORMAL else 3))
    after = np.concatenate(u0)
    after[z["idx"]] = z["val"]
    offs = np.cumsum([0] + [g.size for g in grids])
    u = [after[offs[i]:offs[i + 1]].copy() for i in range(len(grids))]
    return case, tuple(int(v) for v in z["spec"]), u


def coupled_files():
    """solve fixtures of two elliptic variables (load them with load())"""
    return sorted(glob.glob(os.path.join(GOLDEN, "coupled_*.npz")))


def regrid_files():
    """the regrid fixtures"""
    return sorted(glob.glob(os.path.join(GOLDEN, "regrid*.npz")))


def load_regrid(path: str):
    """(old case with the fixture's seeded u and source, new case with zero
    data, (min_lev, order), u and source the reference's regrid left on every
    new grid: the old data on the kept grids below min_lev)"""
    z = np.load(path)
    dim = int(z["dim"])

    def grids(table):
        out = []
        for row in table:
            lev, s0, s1, s2 = (int(v) for v in row[:4])
            out.append(W.Grid(lev, tuple(float(v) for v in row[4:4 + 2 * dim]), (s0, s1, s2)))
        return out
    shape = tuple(int(v) for v in z["base_shape"])
    bbox = tuple(float(v) for v in z["base_bbox"])
    name = str(z["name"])
    og, ng = grids(z["old"]), grids(z["new"])
    old = W.Case(name[:-4] + "_old", W.POISSON, dim, shape, bbox, og, [np.zeros(g.size) for g in og],
                 [np.zeros(g.size) for g in og], W.MGParams())
    W.regrid_data(old, int(z["seed"]))
    new = W.Case(name, W.POISSON, dim, shape, bbox, ng, [np.zeros(g.size) for g in ng],
                 [np.zeros(g.size) for g in ng], W.MGParams())
    min_lev, order = (int(v) for v in z["spec"])
    u, src, off = [], [], 0
    for g in ng:
        if g.level < min_lev:   # kept: the old grid's data
            i = next(i for i, o in enumerate(og) if o.level == g.level and o.shape == g.shape and o.bbox == g.bbox)
            u.append(old.u0[i].copy())
            src.append(old.src[i].copy())
        else:
            u.append(z["u"][off:off + g.size].copy())
            src.append(z["src"][off:off + g.size].copy())
            off += g.size
    return old, new, (min_lev, order), u, src


def load(path: str):
    z = np.load(path)
    grids = []
    for row in z["grids"]:
        lev, s0, s1, s2 = (int(v) for v in row[:4])
        dim = int(z["dim"])
        bbox = tuple(float(v) for v in row[4:4 + 2 * dim])
        grids.append(W.Grid(lev, bbox, (s0, s1, s2)))
    ip = [int(v) for v in z["params"]]
    fp = [float(v) for v in z["fparams"]]
    params = W.MGParams(pre_swp=ip[0], pst_swp=ip[1], max_iter=ip[2], min_iter=ip[3],
                        max_citer=ip[4], min_cwidth=ip[5], restr_u=ip[6], restr_res=ip[7],
                        restr_src=ip[8], interp_order=ip[9], tol=fp[0], crtol=fp[1],
                        w0_r=fp[2], w0_i=fp[3])
    sizes = [g.size for g in grids]
    offs = np.cumsum([0] + sizes)
    split = lambda a: [a[offs[i]:offs[i + 1]].copy() for i in range(len(grids))]  # noqa: E731
    case = W.Case(str(z["name"]), int(z["pde"]), int(z["dim"]),
                  tuple(int(v) for v in z["base_shape"]),
                  tuple(float(v) for v in z["base_bbox"]), grids,
                  split(z["u0"]), split(z["src"]), params)
    if "src1" in z.files and len(z["src1"]):
        case.src_extra = [split(z["src1"])]
    if "min_level" in z.files:
        case.min_level = int(z["min_level"])
    if "u1_0" in z.files and len(z["u1_0"]):   # the second elliptic variable
        case.u_extra = [split(z["u1_0"])]
    masks = []
    off = 0
    for kind, L, idx in z["masks_meta"]:
        mg = [r for r in z["mgh"] if int(r[0]) == L and int(r[1]) == idx][0]
        n = int(mg[2] * mg[3] * mg[4])
        masks.append({"kind": ("bdy", "child")[int(kind)], "L": int(L), "idx": int(idx),
                      "mask": z["masks"][off:off + n].astype(np.float64)})
        off += n
    ref = {
        "iters": int(z["iters"]),
        "hooks": {"kind": z["hook_kind"].astype(np.int32), "L": z["hook_L"].astype(np.int32),
                  "idx": z["hook_idx"].astype(np.int32), "norm": z["hook_norm"]},
        "mgh": [{"L": int(r[0]), "idx": int(r[1]), "shape": (int(r[2]), int(r[3]), int(r[4])),
                 "coarsest": int(r[5]), "bbox": tuple(float(v) for v in r[6:12])}
                for r in z["mgh"]],
        "masks": masks,
        "u": split(z["u"]),
        "gfn": dict(zip(("u", "res", "lop", "rhs", "cmask", "src", "src1", "src2", "src3"),
                        (int(v) for v in z["gfn"]))),
        "ops": z["ops"].astype(np.int64),
        "u_extra": [split(z["u1"])] if "u1" in z.files and len(z["u1"]) else [],
    }
    return case, ref


def finest_residuals(hooks: dict, lf: int) -> np.ndarray:
    """per-V-cycle finest residual (amrd/mg.c:194) from a hook log"""
    k, L, n = hooks["kind"], hooks["L"], hooks["norm"]
    pos = np.nonzero((k == 1) & (L == lf))[0]
    groups, last = [], None
    for p in pos:
        if last is not None and p == last + 1:
            groups[-1].append(p)
        else:
            groups.append([p])
        last = p
    out = np.array([max(float(n[i]) for i in g) for g in groups])
    return out[1::2] if lf > 1 else out


def expand_trace(tr: dict):
    """expands a device trace's periodic-skip markers (kind 2: period in
    'idx', skipped iterations in 'repeat') into the norms the reference
    logs for the skipped coarsest-grid iterations"""
    out = {"kind": [], "L": [], "idx": [], "norm": []}
    for i in range(len(tr["kind"])):
        if tr["kind"][i] != 2:
            for key in ("kind", "L", "idx", "norm"):
                out[key].append(tr[key][i])
            continue
        period, skip, lev = int(tr["idx"][i]), int(tr["repeat"][i]), int(tr["L"][i])
        # the last `period` iterations' records on this level (one per coarsest box)
        recs = []
        j = len(out["kind"]) - 1
        while j >= 0 and out["kind"][j] == 0 and out["L"][j] == lev:
            recs.append(j)
            j -= 1
        recs = recs[::-1]
        nbox = 1
        if recs:
            first_box = out["idx"][recs[-1]]
            nbox = 1
            while nbox < len(recs) and out["idx"][recs[-1 - nbox]] != first_box:
                nbox += 1
        cyc = recs[-period * nbox:]
        for s in range(skip):
            for jj in cyc[(s % period) * nbox:(s % period + 1) * nbox]:
                for key in ("kind", "L", "idx", "norm"):
                    out[key].append(out[key][jj])
    return {k: np.array(v) for k, v in out.items()}
