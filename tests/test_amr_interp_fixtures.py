"""The AMR-hierarchy interpolation fixtures (made from the reference's own
PAMR_interp / PAMR_AMR_bdy_interp by tests/golden/make_golden.py) load on the
CPU: the seeded u regenerates, every changed point lies on a grid of the
fine level, and a boundary band changes fewer points than the whole
overlap of the same transfer would."""
import numpy as np
import pytest

import golden_cases as G


@pytest.mark.parametrize("path", G.interp_files(), ids=lambda p: p.split("/")[-1][:-4])
def test_fixture_changes_only_the_fine_level(path):
    case, (lc, width, order), u = G.load_interp(path)
    assert order in (2, 4) and width >= 0
    changed = [int(np.sum(a != b)) for a, b in zip(u, case.u0)]
    assert sum(changed) > 0
    for g, n in zip(case.grids, changed):
        assert n == 0 or g.level == lc + 1
        assert n <= g.size


def test_there_are_band_and_overlap_fixtures():
    specs = [G.load_interp(p)[1] for p in G.interp_files()]
    assert any(w == 0 for _, w, _ in specs) and any(w > 0 for _, w, _ in specs)
    assert {o for _, _, o in specs} == {2, 4}
