"""The oracle port (oracle/port/mg_port.c) against the golden fixtures made by
the compiled reference: same V-cycle count, bit-identical solution, and the
same sequence of hook calls with bit-identical norms."""
import numpy as np
import pytest

import golden_cases as G
from oracle import portrun, refrun
from pamr_amrd_gb300 import workloads as W


@pytest.mark.parametrize("path", G.files(), ids=lambda p: p.split("/")[-1][:-4])
def test_port_matches_reference_fixture(path):
    case, ref = G.load(path)
    p = portrun.solve(case, hook_cap=len(ref["hooks"]["kind"]) + 10)
    assert p["iters"] == ref["iters"]
    for a, b in zip(p["u"], ref["u"]):
        assert np.array_equal(a, b)
    h, rh = p["hooks"], ref["hooks"]
    assert len(h["kind"]) == len(rh["kind"])
    for k in ("kind", "L", "idx"):
        assert np.array_equal(h[k], rh[k])
    assert np.array_equal(h["norm"], rh["norm"])


@pytest.mark.skipif(not refrun.available(), reason="reference sources not built here")
@pytest.mark.parametrize("seed", [5, 6])
def test_port_matches_reference_live(seed):
    case = W.poisson2d_uneven(seed=seed, n=33, levels=3, min_boxes=3, max_boxes=6, min_side=5,
                              max_side=17)
    ref = refrun.run_reference(case)
    p = portrun.solve(case)
    assert p["iters"] == ref["iters"]
    for a, b in zip(p["u"], ref["u"]):
        assert np.array_equal(a, b)


def test_amplitudes_beyond_existence_diverge_in_port():
    """the conformal workload uses amplitudes U(0,0.005): ten times larger
    (compactness of order one) the reference FAS has no solution to find"""
    orig = W._gaussians
    try:
        W._gaussians = lambda g, d, blobs: orig(g, d, [(a * 10, w, c) for (a, w, c) in blobs])
        case = W.conformal3d(33, 17, seed=0)
    finally:
        W._gaussians = orig
    case.params.max_iter = 6
    p = portrun.solve(case)
    assert not (p["res"][-1] <= case.params.tol)


LIVE_FAMILIES = {
    "conformal3d_17_9_s11": lambda: W.conformal3d(17, 9, seed=11),
    "conformal3d_33_17_s12": lambda: W.conformal3d(33, 17, seed=12),
    "poisson3d_17_s13": lambda: W.poisson3d(17, seed=13),
    "poisson2d_33_s14": lambda: W.poisson2d(33, seed=14),
    "lapse2d_bo_33_L3_s15": lambda: W.lapse2d_bo(33, seed=15, levels=3, step=77),
    "uneven_s16": lambda: W.poisson2d_uneven(seed=16, n=33, levels=4, min_boxes=2, max_boxes=5,
                                             min_side=5, max_side=17),
    "conformal3d_65_33_s21": lambda: W.conformal3d(65, 33, seed=21),
    "poisson3d_33_s24": lambda: W.poisson3d(33, seed=24),
    "lapse2d_bo_65_L4_s22": lambda: W.lapse2d_bo(65, seed=22, levels=4, step=333),
    "uneven65_s23": lambda: W.poisson2d_uneven(seed=23, n=65, levels=5, min_boxes=8, max_boxes=16),
}


@pytest.mark.skipif(not refrun.available(), reason="reference sources not built here")
@pytest.mark.parametrize("name", sorted(LIVE_FAMILIES))
def test_port_matches_reference_live_families(name):
    """every operator and hierarchy family the workloads build, on seeds no
    fixture uses: the port against the compiled reference, hook for hook"""
    case = LIVE_FAMILIES[name]()
    ref = refrun.run_reference(case)
    p = portrun.solve(case, hook_cap=len(ref["hooks"]) + 10)
    assert p["iters"] == ref["iters"]
    for a, b in zip(p["u"], ref["u"]):
        assert np.array_equal(a, b)
    h, rh = p["hooks"], ref["hooks"]
    assert len(h["kind"]) == len(rh)
    for k in ("kind", "L", "idx", "norm"):
        assert np.array_equal(h[k], rh[k])
