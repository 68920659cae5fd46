"""Interpolation on the AMR hierarchy on the GPU (pgb_amr_interp: the
transfer PAMR_interp / PAMR_AMR_bdy_interp perform) against the reference's
own results (tests/golden/amr_interp_*), bit for bit on every grid: 2-D
uneven and 3-D nested hierarchies, orders 2 and 4, whole overlap and
boundary bands of width 1-3."""
import numpy as np
import pytest

import golden_cases as G
from pamr_amrd_gb300.solver import Solver

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", G.interp_files(), ids=lambda p: p.split("/")[-1][:-4])
def test_amr_interp_matches_reference(path):
    case, (lc, width, order), want = G.load_interp(path)
    s = Solver(case)
    s.set_inputs()
    s.amr_interp(lc, width, order)
    got = s.get_u()
    s.close()
    for g, (a, b) in enumerate(zip(got, want)):
        assert np.array_equal(a, b), (g, int(np.sum(a != b)))
