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
