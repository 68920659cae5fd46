"""Host-side bookkeeping of libpamr_gb300 (no GPU needed): the MG hierarchy,
the cmask arrays and every transfer op must equal the reference's, bit for
bit (golden fixtures from the compiled reference)."""
import numpy as np
import pytest

import bookkeeping as BK
import golden_cases as G
from oracle import refrun
from pamr_amrd_gb300 import workloads as W
from pamr_amrd_gb300.solver import PgbError, Solver


def _check_case(case, ref):
    s = Solver(case, host_only=True)
    nb = sum(s.level_nbox(L) for L in range(1, s.num_levels() + 1))
    assert nb == len(ref["mgh"])
    for r in ref["mgh"]:
        b = s.box_info(r["L"], r["idx"])
        assert b["shape"] == r["shape"]
        assert b["coarsest"] == r["coarsest"]
        assert all(b["bbox"][k] == r["bbox"][k] for k in range(2 * case.dim))
    for m in ref["masks"]:
        assert np.array_equal(s.cmask(m["L"], m["idx"], m["kind"]), m["mask"])
    exp = BK.expected_calls(s, BK.reference_gfns(ref), ref["iters"], case.params.pre_swp,
                            case.params.pst_swp)
    assert exp.shape == ref["ops"].shape
    assert np.array_equal(exp, ref["ops"])


@pytest.mark.parametrize("path", G.files(), ids=lambda p: p.split("/")[-1][:-4])
def test_plans_match_reference_fixture(path):
    case, ref = G.load(path)
    _check_case(case, ref)


@pytest.mark.skipif(not refrun.available(), reason="reference sources not built here")
@pytest.mark.parametrize("seed", [7, 8, 9])
def test_plans_match_reference_live(seed):
    case = W.poisson2d_uneven(seed=seed, n=65, levels=4, min_boxes=4, max_boxes=12, min_side=9,
                              max_side=41)
    ref = refrun.run_reference(case, log_ops=True)
    ref["ops"] = ref["ops"].astype(np.int64)
    _check_case(case, ref)


PLAN_FAMILIES = {
    "conformal3d_33_17_s31": lambda: W.conformal3d(33, 17, seed=31),
    "poisson3d_17_s32": lambda: W.poisson3d(17, seed=32),
    "lapse2d_bo_65_L4_s33": lambda: W.lapse2d_bo(65, seed=33, levels=4, step=5),
    "uneven65_L5_s34": lambda: W.poisson2d_uneven(seed=34, n=65, levels=5, min_boxes=8, max_boxes=16),
}


@pytest.mark.skipif(not refrun.available(), reason="reference sources not built here")
@pytest.mark.parametrize("name", sorted(PLAN_FAMILIES))
def test_plans_match_reference_live_families(name):
    """the hierarchy, both cmask arrays and the whole m_util_r8 call sequence
    of a solve against the compiled reference, for every hierarchy family"""
    case = PLAN_FAMILIES[name]()
    ref = refrun.run_reference(case, log_ops=True)
    ref["ops"] = ref["ops"].astype(np.int64)
    _check_case(case, ref)


def test_invalid_inputs_are_errors_not_exits():
    case = W.poisson2d(17)
    case.params.interp_order = 3
    with pytest.raises(PgbError):
        Solver(case, host_only=True)
    case = W.poisson2d(17)
    case.grids[0] = W.Grid(0, case.grids[0].bbox, case.grids[0].shape)
    with pytest.raises(PgbError):
        Solver(case, host_only=True)


@pytest.mark.parametrize("make", [lambda: W.conformal3d(65, 33, seed=3),
                                  lambda: W.poisson2d_uneven(seed=4, n=129, levels=5, min_boxes=8,
                                                             max_boxes=16),
                                  lambda: W.lapse2d_bo(65, seed=5, levels=4, step=120)]
                         + [lambda p=p: G.load(p)[0] for p in G.files()],
                         ids=["c3d65", "uneven129", "lapse65"] + [p.split("/")[-1][:-4] for p in G.files()])
def test_child_covered_points_are_restricted(make):
    """Every child-covered point (cmask_child on) of a level is written by
    the restriction of res into it, so the FAS right-hand side never reads
    a res value of an earlier cycle (the mixed form skips the clear of res
    on levels whose residual is restricted from its FP32 copy)."""
    s = Solver(make(), host_only=True)
    for L in range(1, s.num_levels()):
        ops = s.plan(3, L)
        for idx in range(s.level_nbox(L)):
            sh = s.box_info(L, idx)["shape"]
            cm = s.cmask(L, idx, "child").reshape(sh[2], sh[1], sh[0]) != 0
            covered = np.zeros_like(cm)
            for r in ops:
                if r[2] != L or r[3] != idx or r[14 + 2] == 0:   # dst level/box, op of res
                    continue
                i2, j2, k2, ni, nj, nk = r[7:13]
                covered[k2 - 1:k2 - 1 + nk, j2 - 1:j2 - 1 + nj, i2 - 1:i2 - 1 + ni] = True
            assert not np.any(cm & ~covered), (L, idx)
    s.close()
