"""The regrid fixtures (tests/golden/regrid*): what the reference's
PAMR_compose_hierarchy (init_new_cgh, src/gh.c:934-1045) left on the grids
of a new hierarchy. Checked here on the CPU for the transfer semantics the
GPU regrid must reproduce: a new grid identical to an old one that owned
its whole region holds the old data bit for bit (the copy from the old
level overwrites the interpolation), and every point of every new grid was
reached (no zero left from the new hierarchy's initial data)."""
import numpy as np
import pytest

import golden_cases as G


def _owns_all(case, i):
    """old grid i is not overlapped by an earlier grid of its level (PAMR's
    build_owned_gsl gives overlaps to the earlier grid)"""
    g = case.grids[i]
    for o in case.grids[:i]:
        if o.level != g.level:
            continue
        if all(o.bbox[2 * d] < g.bbox[2 * d + 1] and g.bbox[2 * d] < o.bbox[2 * d + 1] for d in range(case.dim)):
            return False
    return True


@pytest.mark.parametrize("path", G.regrid_files(), ids=lambda p: p.split("/")[-1][:-4])
def test_regrid_fixture_semantics(path):
    old, new, (min_lev, order), u, src = G.load_regrid(path)
    assert len(u) == len(new.grids)
    kept = 0
    for j, g in enumerate(new.grids):
        assert np.all(np.isfinite(u[j])) and np.all(u[j] != 0.0)
        assert np.all(src[j] != 0.0)
        for i, o in enumerate(old.grids):
            if o.level == g.level and o.shape == g.shape and o.bbox == g.bbox and _owns_all(old, i) \
                    and g.level >= min_lev:
                assert np.array_equal(u[j], old.u0[i])
                assert np.array_equal(src[j], old.src[i])
                kept += 1
    assert kept >= 1
