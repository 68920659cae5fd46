"""Generates the golden fixtures in tests/golden/ by running the reference's
own multigrid solve (oracle/_ref/ref_mg, compiled from the reference's C
sources by oracle/build_ref.sh) on small seeded cases.

The coupled_* fixtures are solve fixtures of two elliptic variables solved
together (the second variable's initial and final values beside the first).
The regrid_* fixtures store an old and a new grid list, the seed of the old
grids' random u and source, (min_lev, order), and u and the source the
reference's PAMR_compose_hierarchy left on the new grids it recomposed.
The amr_interp_* fixtures store a case's grids, the seed of its random u,
the transfer (AMR level, boundary width, order) and the points the
reference's PAMR_interp / PAMR_AMR_bdy_interp changed, with their values. The others store the case (grids,
parameters, initial u and source) and what the reference's solve produced: V-cycle count, every relax/residual/L_op hook
call with its norm, the MG hierarchy, the cmask arrays, the final u on every
grid and the m_util_r8 call log of the whole solve. Cases with an
application operator (two sources) or an MG hierarchy built from an AMR
level above the base also store the second source and that level.

usage: python tests/golden/make_golden.py [--all]   (needs oracle/_ref/ref_mg)
Writes the fixtures that are missing; --all rewrites every one.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import refrun  # noqa: E402
from pamr_amrd_gb300 import workloads as W  # noqa: E402


def cases():
    return [
        W.poisson2d(17, seed=0),
        W.poisson2d(33, seed=1),
        W.conformal3d(17, 9, seed=0),
        W.conformal3d(17, 9, seed=3, params=W.MGParams(min_cwidth=5, pre_swp=3, pst_swp=1)),
        W.poisson2d_uneven(seed=1, n=33, levels=3, min_boxes=2, max_boxes=4, min_side=5,
                           max_side=17),
        W.poisson2d_uneven(seed=2, n=65, levels=4, min_boxes=3, max_boxes=8, min_side=9,
                           max_side=33),
        W.lapse2d_bo(17, seed=0, levels=3),
        W.lapse2d_bo(17, seed=1, levels=3, step=100),
        # an application operator with two sources (the nbs potential)
        W.nbs3d(17, 9, seed=0),
        W.nbs2d_uneven(seed=1, n=33, levels=3, min_boxes=2, max_boxes=4, min_side=5, max_side=17),
        # MG hierarchies built from an AMR level above the base
        # (solve_elliptics(L, ...) with L > 1; L = finest as at amrd/evolve.c:454)
        W.with_min_level(W.lapse2d_bo(33, seed=2, levels=3, step=40), 2),
        W.with_min_level(W.lapse2d_bo(33, seed=3, levels=3, step=80), 3),
        W.with_min_level(W.poisson2d_uneven(seed=2, n=65, levels=4, min_boxes=3, max_boxes=8,
                                            min_side=9, max_side=33), 3),
    ]


def coupled_cases():
    """two elliptic variables solved together (workloads.VAR_OPERATORS[COUPLED])
    on a single grid, nested boxes in 3-D and an uneven multi-box hierarchy"""
    return [
        W.coupled_from(W.poisson2d(33, seed=0), seed=1),
        W.coupled_from(W.conformal3d(17, 9, seed=0), seed=2),
        W.coupled_from(W.poisson2d_uneven(seed=1, n=33, levels=3, min_boxes=2, max_boxes=4, min_side=5,
                                          max_side=17), seed=3),
    ]


def dropin_cases():
    """(case, mode, arg, level) of the drop-in application fixtures
    (tests/dropin/nbs_app.c built over the reference's PAMR/AMRD with
    amrd/mg.c): mode 0 solve_elliptics(level, 1, 0); mode 1 PAMR_build_mgh
    of the finest level and `arg` vcycle calls with the finest sources
    changed between them"""
    small = dict(n=33, levels=3, min_boxes=2, max_boxes=4, min_side=5, max_side=17)
    return [
        (W.nbs2d_uneven(seed=1, **small), 0, 0, 1),
        (W.nbs3d(17, 9, seed=0), 0, 0, 1),
        (W.nbs2d_uneven(seed=2, **small), 0, 0, 2),
        (W.nbs2d_uneven(seed=1, **small), 1, 4, 0),
        (W.nbs3d(17, 9, seed=4, levels=3), 1, 3, 0),
        # two elliptic variables solved together (the coupled pair)
        (W.coupled_from(W.nbs2d_uneven(seed=1, **small), seed=4), 0, 0, 1),
        (W.coupled_from(W.nbs3d(17, 9, seed=0), seed=5), 0, 0, 1),
        # the coupled pair through vcycle on the finest level's MG hierarchy
        (W.coupled_from(W.nbs2d_uneven(seed=1, **small), seed=6), 1, 3, 0),
        (W.coupled_from(W.nbs3d(17, 9, seed=4, levels=3), seed=7), 1, 3, 0),
        (W.coupled_from(W.nbs3d(17, 9, seed=4, levels=3), seed=7), 1, 1, 0),
    ]


def save_dropin(case, mode, arg, level, out, path):
    """the case (as save() stores it) and what the application wrote: cycle
    count, residuals, u and cmask of every AMR grid in PAMR order"""
    from tests.dropin import dropin as D
    res = out["res"] if mode == 1 else D.finest_residuals(out)
    grids = np.array([[g.level] + list(g.shape) + list(g.bbox) + [0.0] * (6 - len(g.bbox))
                      for g in case.grids])
    p = case.params
    og = np.array([[g["level"], *g["shape"], *g["bbox"]] for g in out["grids"]])
    np.savez_compressed(
        path, name=np.array(case.name), pde=case.pde, dim=case.dim,
        base_shape=np.array(case.base_shape), base_bbox=np.array(case.base_bbox), grids=grids,
        u0=np.concatenate(case.u0), src=np.concatenate(case.src), src1=np.concatenate(case.source(1)),
        params=np.array([p.pre_swp, p.pst_swp, p.max_iter, p.min_iter, p.max_citer,
                         p.min_cwidth, p.restr_u, p.restr_res, p.restr_src, p.interp_order]),
        fparams=np.array([p.tol, p.crtol, p.w0_r, p.w0_i]),
        mode=mode, arg=arg, level=level, iters=out["iters"], res=res, out_grids=og,
        out_u=np.concatenate([g["u"] for g in out["grids"]]),
        out_cmask=np.concatenate([g["cmask"] for g in out["grids"]]).astype(np.uint8),
        # the second elliptic variable of a coupled case: initial, and as written
        u1_0=np.concatenate(case.var(1)) if case.nvar > 1 else np.zeros(0),
        out_w=np.concatenate([g["w"] for g in out["grids"]]) if case.nvar > 1 else np.zeros(0))


def interp_cases():
    """(case with seeded random u, (lc, AMR boundary width, order)) for the
    AMR-hierarchy interpolation fixtures"""
    out = []
    for make, specs in (
            (lambda: W.poisson2d_uneven(seed=1, n=33, levels=3, min_boxes=2, max_boxes=4, min_side=5,
                                        max_side=17), [(1, 0, 2), (1, 2, 4), (2, 0, 4), (2, 1, 2)]),
            (lambda: W.poisson2d_uneven(seed=2, n=65, levels=4, min_boxes=3, max_boxes=8, min_side=9,
                                        max_side=33), [(2, 0, 4), (3, 2, 2), (3, 3, 4)]),
            (lambda: W.conformal3d(17, 9, seed=0), [(1, 0, 2), (1, 1, 4), (2, 2, 4)])):
        for spec in specs:
            c = make()
            seed = len(out) + 11
            c.u0 = interp_u0(c, seed)
            out.append((c, spec, seed))
    return out


def interp_u0(case, seed):
    """the seeded random u the interpolation fixtures start from"""
    rng = np.random.default_rng(seed)
    return [rng.standard_normal(g.size) for g in case.grids]


def save_interp(case, spec, seed, u_after, path):
    """the case's grids, the seed of u, the transfer, and the points the
    reference's interpolation changed (index into the concatenated grids, value)"""
    grids = np.array([[g.level] + list(g.shape) + list(g.bbox) + [0.0] * (6 - len(g.bbox))
                      for g in case.grids])
    before, after = np.concatenate(case.u0), np.concatenate(u_after)
    idx = np.nonzero(after != before)[0].astype(np.int32)
    np.savez_compressed(path, name=np.array(case.name), pde=case.pde, dim=case.dim,
                        base_shape=np.array(case.base_shape), base_bbox=np.array(case.base_bbox),
                        grids=grids, seed=seed, spec=np.array(spec), idx=idx, val=after[idx])


def regrid_cases():
    """(old case with seeded random u and source, new case, data seed,
    (min_lev, order)) for the regrid fixtures"""
    out = []
    for seed, dim, n, finer, order in ((1, 2, 33, False, 2), (2, 2, 33, True, 4), (3, 3, 17, False, 2),
                                       (4, 3, 17, True, 4)):
        old, new = W.regrid_pair(seed=seed, dim=dim, n=n, finer=finer)
        W.regrid_data(old, 100 + seed)
        out.append((old, new, 100 + seed, (2, order)))
    return out


def save_regrid(old, new, seed, spec, ref, path):
    """both grid lists, the data seed, (min_lev, order), and u and the source
    the reference's regrid left on every new grid of level >= min_lev (in the
    new case's grid order); the grids below keep the old data"""
    def table(case):
        return np.array([[g.level] + list(g.shape) + list(g.bbox) + [0.0] * (6 - len(g.bbox))
                         for g in case.grids])
    us, ss = [], []
    for g in new.grids:
        if g.level < spec[0]:
            continue
        hit = [r for r in ref["regrid"] if r["L"] == g.level and r["shape"] == g.shape and
               np.allclose(r["bbox"][:2 * new.dim], g.bbox, rtol=0, atol=1e-12)]
        assert len(hit) == 1, (g, len(hit))
        us.append(hit[0]["u"])
        ss.append(hit[0]["src"][0])
    np.savez_compressed(path, name=np.array(new.name), dim=new.dim, base_shape=np.array(new.base_shape),
                        base_bbox=np.array(new.base_bbox), old=table(old), new=table(new), seed=seed,
                        spec=np.array(spec), u=np.concatenate(us), src=np.concatenate(ss))


def save(case, ref, path):
    p = case.params
    grids = np.array([[g.level] + list(g.shape) + list(g.bbox) + [0.0] * (6 - len(g.bbox))
                      for g in case.grids])
    masks_meta = np.array([[0 if m["kind"] == "bdy" else 1, m["L"], m["idx"]]
                           for m in ref["masks"]], dtype=np.int32)
    masks = np.concatenate([m["mask"] for m in ref["masks"]]).astype(np.uint8)
    mgh = np.array([[r["L"], r["idx"], *r["shape"], r["coarsest"], *r["bbox"]]
                    for r in ref["mgh"]])
    h = ref["hooks"]
    np.savez_compressed(
        path,
        name=np.array(case.name), pde=case.pde, dim=case.dim,
        base_shape=np.array(case.base_shape), base_bbox=np.array(case.base_bbox),
        grids=grids,
        u0=np.concatenate(case.u0), src=np.concatenate(case.src),
        src1=np.concatenate(case.source(1)) if case.nsrc > 1 else np.zeros(0),
        min_level=case.min_level,
        params=np.array([p.pre_swp, p.pst_swp, p.max_iter, p.min_iter, p.max_citer,
                         p.min_cwidth, p.restr_u, p.restr_res, p.restr_src, p.interp_order]),
        fparams=np.array([p.tol, p.crtol, p.w0_r, p.w0_i]),
        iters=ref["iters"],
        hook_kind=h["kind"].astype(np.int8), hook_L=h["L"].astype(np.int8),
        hook_idx=h["idx"].astype(np.int16), hook_norm=h["norm"],
        mgh=mgh, masks_meta=masks_meta, masks=masks,
        u=np.concatenate(ref["u"]),
        gfn=np.array([ref["gfn"][k] for k in refrun.GFN_KEYS if k in ref["gfn"]]),
        ops=ref["ops"].astype(np.int16) if len(ref["ops"]) else np.zeros((0, 34), np.int16),
        # the second elliptic variable of a coupled case: initial and final values
        u1_0=np.concatenate(case.var(1)) if case.nvar > 1 else np.zeros(0),
        u1=np.concatenate(ref["u_extra"]) if case.nvar > 1 else np.zeros(0),
    )


def main():
    if not refrun.available():
        raise SystemExit("oracle/_ref/ref_mg missing: run oracle/build_ref.sh first")
    for c in cases():
        path = os.path.join(HERE, f"{c.name}__{len(c.grids)}g_{c.params.min_cwidth}cw.npz")
        if os.path.exists(path) and "--all" not in sys.argv:
            continue
        ref = refrun.run_reference(c, log_ops=True)
        save(c, ref, path)
        print(f"{os.path.basename(path)}: {ref['iters']} V-cycles, {len(ref['hooks'])} hook calls, "
              f"{len(ref['ops'])} m_util_r8 calls, {os.path.getsize(path) // 1024} KiB")
    for c in coupled_cases():
        path = os.path.join(HERE, f"{c.name}__{len(c.grids)}g_{c.params.min_cwidth}cw.npz")
        if os.path.exists(path) and "--all" not in sys.argv:
            continue
        ref = refrun.run_reference(c)
        save(c, ref, path)
        print(f"{os.path.basename(path)}: {ref['iters']} V-cycles, {len(ref['hooks'])} hook calls, "
              f"{os.path.getsize(path) // 1024} KiB")
    from tests.dropin import dropin as D
    for c, mode, arg, level in dropin_cases():
        path = os.path.join(HERE, f"dropin_{c.name}_m{mode}_a{arg}_L{level}.npz")
        if os.path.exists(path) and "--all" not in sys.argv:
            continue
        out = D.run(D.REF_APP, c, mode=mode, arg=arg, level=level)
        save_dropin(c, mode, arg, level, out, path)
        print(f"{os.path.basename(path)}: {out['iters']} cycles, {os.path.getsize(path) // 1024} KiB")
    for c, spec, seed in interp_cases():
        lc, w, o = spec
        path = os.path.join(HERE, f"amr_interp_{c.name}_L{lc}_w{w}_o{o}.npz")
        if os.path.exists(path) and "--all" not in sys.argv:
            continue
        ref = refrun.run_reference(c, amr_interp=spec)
        save_interp(c, spec, seed, ref["u"], path)
        changed = sum(int(np.sum(a != b)) for a, b in zip(ref["u"], c.u0))
        print(f"{os.path.basename(path)}: {changed} points interpolated, {os.path.getsize(path) // 1024} KiB")

    for old, new, seed, spec in regrid_cases():
        path = os.path.join(HERE, f"{new.name[:-4]}_m{spec[0]}_o{spec[1]}.npz")
        if os.path.exists(path) and "--all" not in sys.argv:
            continue
        ref = refrun.run_reference(old, regrid=(new, spec[0], spec[1]))
        save_regrid(old, new, seed, spec, ref, path)
        print(f"{os.path.basename(path)}: {len(ref['regrid'])} grids after the regrid, "
              f"{os.path.getsize(path) // 1024} KiB")


if __name__ == "__main__":
    main()
