"""The small-level kernel of the mixed form: the V-cycle's passes over the MG
levels of at most 6000 points (residual, restriction, FAS right-hand side,
colour passes, defect carry, update, coarsest-grid loop, coarse-grid
correction, interpolation) run as the steps of one thread-block cluster
launch instead of one launch each. Every step runs the body of the kernel it
replaces, so a solve with it (PGB_TAIL=1; it is off by default) gives the same
V-cycles, norms and solution bit for bit as one without it. Both run with the default launch
shapes (PGB_AUTOTUNE=0), which is what makes the comparison bit for bit: the
autotuner's tile depths move a few points between the fresh and the carried
FP32 defect."""
import numpy as np
import pytest

from pamr_amrd_gb300 import workloads as W
from pamr_amrd_gb300.solver import Solver

pytestmark = pytest.mark.gpu

CASES = {
    "c3d65": lambda: W.conformal3d(65, 33, seed=1),
    "c3d129": lambda: W.conformal3d(129, 65, seed=0),
    "p3d65": lambda: W.poisson3d(65, seed=2),
    "p3d129": lambda: W.poisson3d(129, seed=3),
    "p2d129": lambda: W.poisson2d(129, seed=0),
    "lapse129": lambda: W.lapse2d_bo(129, seed=1, levels=4, step=40),
    "uneven2d": lambda: W.poisson2d_uneven(seed=1, levels=4, min_boxes=4, max_boxes=8),
}


def _run(monkeypatch, case, env):
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    try:
        s = Solver(case)
        out = []
        for _ in range(2):
            s.set_inputs()
            r = s.solve()
            out.append((r["iters"], r["res"], s.get_u()))
        tail = s.tail_levels()
        modes = [s.level_tuning(L)[1] for L in range(2, s.num_levels() + 1)]
        s.close()
    finally:
        for k in env:
            monkeypatch.delenv(k)
    return out, tail, modes


@pytest.mark.parametrize("mode", ["cluster", "grid", "mini"])
@pytest.mark.parametrize("name", list(CASES))
def test_small_level_kernel_changes_no_bits(monkeypatch, name, mode):
    case = CASES[name]()
    case.params.precision = 1
    env = {"PGB_AUTOTUNE": "0", "PGB_TAIL": "mini" if mode == "mini" else "1"}
    if mode == "grid":
        env["PGB_TAIL_GRID"] = "1"
    with_tail, tail, modes = _run(monkeypatch, case, env)
    without, tail0, modes0 = _run(monkeypatch, case, {"PGB_AUTOTUNE": "0"})
    assert tail0 == (0, 0) and 8 not in modes0
    # levels of one box each, small enough for the mode (mini: at most 1500 points)
    if name in (("p3d65", "p3d129", "p2d129") if mode == "mini" else ("c3d65", "p3d65", "p3d129", "p2d129", "lapse129")):
        assert tail[0] >= 2 and tail[1] >= 1, tail
    # the levels it runs report sweep mode 8, the others keep theirs
    assert modes[: max(tail[0] - 1, 0)] == [8] * max(tail[0] - 1, 0), (tail, modes)
    assert 8 not in modes[max(tail[0] - 1, 0):]
    for (i1, r1, u1), (i2, r2, u2) in zip(with_tail, without):
        assert i1 == i2
        assert np.array_equal(r1, r2), np.max(np.abs(r1 - r2))
        for a, b in zip(u1, u2):
            assert np.array_equal(a, b), float(np.max(np.abs(a - b)))


def test_small_level_kernel_in_the_host_loop_and_direct_launches(monkeypatch):
    """the recorded program is the same whether the V-cycle is captured in
    the device loop's graph, replayed one graph per cycle, or launched
    directly every cycle (PGB_NO_GRAPH=1)"""
    case = W.poisson3d(65, seed=5)
    case.params.precision = 1
    ref, tail, _ = _run(monkeypatch, case, {"PGB_AUTOTUNE": "0", "PGB_TAIL": "1"})
    assert tail[0] >= 2
    for env in ({"PGB_HOST_LOOP": "1"}, {"PGB_NO_GRAPH": "1", "PGB_HOST_LOOP": "1"}):
        out, _, _ = _run(monkeypatch, case, dict(env, PGB_AUTOTUNE="0", PGB_TAIL="1"))
        for (i1, r1, u1), (i2, r2, u2) in zip(out, ref):
            assert i1 == i2 and np.array_equal(r1, r2)
            for a, b in zip(u1, u2):
                assert np.array_equal(a, b)
