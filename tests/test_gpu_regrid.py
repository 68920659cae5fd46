"""Regrid on the GPU (pgb_regrid: PAMR_compose_hierarchy's transfer onto a
new hierarchy, init_new_cgh src/gh.c:934-1045) against the reference's own
results (tests/golden/regrid*): u and the source on every grid of the new
hierarchy, bit for bit, in 2-D and 3-D, interpolation orders 2 and 4, with
and without a new finest level; the old solver is left unchanged."""
import numpy as np
import pytest

import golden_cases as G
from pamr_amrd_gb300.solver import PgbError, Solver

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", G.regrid_files(), ids=lambda p: p.split("/")[-1][:-4])
def test_regrid_matches_reference(path):
    old, new, (min_lev, order), u_ref, src_ref = G.load_regrid(path)
    so = Solver(old)
    so.set_inputs()
    sn = Solver(new)
    sn.set_inputs()
    sn.regrid_from(so, order=order, min_level=min_lev)
    u = sn.get_u()
    src = sn.get_sources()[0]
    for j in range(len(new.grids)):
        assert np.array_equal(u[j], u_ref[j]), (j, float(np.max(np.abs(u[j] - u_ref[j]))))
        assert np.array_equal(src[j], src_ref[j]), j
    for a, b in zip(so.get_u(), old.u0):   # the source hierarchy is only read
        assert np.array_equal(a, b)
    so.close()
    sn.close()


def test_regrid_rejects_bad_arguments():
    old, new, _, _, _ = G.load_regrid(G.regrid_files()[0])
    so, sn = Solver(old), Solver(new)
    with pytest.raises(PgbError):
        sn.regrid_from(so, order=3)
    with pytest.raises(PgbError):
        sn.regrid_from(sn)
    so.close()
    sn.close()
