"""Two elliptic variables solved together (AMRD_num_elliptic_vars = 2,
amrd/mg.c:248-355; operator pair workloads.VAR_OPERATORS[COUPLED]) on the
GPU, FP64 form, against the compiled reference's own solves of the same
cases (tests/golden/coupled_*, its hooks handling both variables point by
point): the same V-cycle count, both variables bit-identical on every grid,
and every relax/residual norm within 1e-12 relative (summation order
only)."""
import numpy as np
import pytest

import golden_cases as G
from pamr_amrd_gb300.solver import Solver

pytestmark = pytest.mark.gpu

NORM_RTOL = 1e-12


@pytest.mark.parametrize("path", G.coupled_files(), ids=lambda p: p.split("/")[-1][:-4])
def test_coupled_matches_reference_fixture(path):
    case, ref = G.load(path)
    assert case.nvar == 2
    s = Solver(case)
    s.set_inputs()
    s.trace_enable(400000)
    r = s.solve()
    vals = s.get_vars()
    tr = G.expand_trace(s.trace_fetch())
    s.close()
    assert r["iters"] == ref["iters"]
    for a, b in zip(vals[0], ref["u"]):
        assert np.array_equal(a, b)
    for a, b in zip(vals[1], ref["u_extra"][0]):
        assert np.array_equal(a, b)
    h = ref["hooks"]
    keep = h["kind"] != 2                      # L_op returns no norm
    assert len(tr["kind"]) == int(keep.sum())
    assert np.array_equal(tr["kind"], h["kind"][keep])
    assert np.array_equal(tr["L"], h["L"][keep])
    rel = np.abs(tr["norm"] - h["norm"][keep]) / np.maximum(np.abs(h["norm"][keep]), 1e-300)
    assert float(np.max(rel)) < NORM_RTOL
