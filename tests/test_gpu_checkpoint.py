"""Checkpoint and restart of the device hierarchy (pgb_checkpoint_save /
pgb_checkpoint_load): a solver restored from a checkpoint taken in the
middle of the Berger-Oliger lapse sequence holds the saved lapse bit for
bit and continues the sequence exactly as the original; a checkpoint of
another hierarchy, or a file that is not a checkpoint, is refused and
leaves the solver's data as it was."""
import numpy as np
import pytest

from pamr_amrd_gb300 import workloads as W
from pamr_amrd_gb300.solver import PgbError, Solver

pytestmark = pytest.mark.gpu


def _step(s, k, u):
    c = W.lapse2d_bo(33, seed=6, levels=4, step=k, steps=8)
    s.set_inputs(u if u is not None else c.u0, c.src)
    r = s.solve()
    return r, s.get_u()


def test_restart_continues_bit_for_bit(tmp_path):
    case = W.lapse2d_bo(33, seed=6, levels=4, steps=8)
    a = Solver(case)
    _, u = _step(a, 0, None)
    _, u = _step(a, 1, u)
    path = str(tmp_path / "lapse.ckpt")
    a.checkpoint_save(path)
    ra, ua = _step(a, 2, u)
    b = Solver(case)
    b.checkpoint_load(path)
    ub = b.get_u()
    for x, y in zip(ub, u):
        assert np.array_equal(x, y)
    rb, ub = _step(b, 2, ub)
    assert ra["iters"] == rb["iters"]
    for x, y in zip(ua, ub):
        assert np.array_equal(x, y)
    a.close()
    b.close()


def test_mismatched_or_foreign_files_are_refused(tmp_path):
    small = Solver(W.lapse2d_bo(33, seed=6, levels=3, steps=8))
    small.set_inputs()
    path = str(tmp_path / "small.ckpt")
    small.checkpoint_save(path)
    other = Solver(W.lapse2d_bo(33, seed=6, levels=4, steps=8))
    other.set_inputs()
    before = other.get_u()
    with pytest.raises(PgbError):
        other.checkpoint_load(path)
    junk = tmp_path / "junk.ckpt"
    junk.write_bytes(b"not a checkpoint at all")
    with pytest.raises(PgbError):
        other.checkpoint_load(str(junk))
    for x, y in zip(other.get_u(), before):
        assert np.array_equal(x, y)
    small.close()
    other.close()


def test_several_variables_restart_bit_for_bit(tmp_path):
    """a solver of two coupled elliptic variables (reference fixture case)
    checkpointed after three V-cycles: the restored solver holds both
    variables bit for bit and finishes the solve exactly as the original"""
    import golden_cases as G
    case, _ = G.load(G.coupled_files()[0])
    assert case.nvar == 2
    a = Solver(case)
    a.set_inputs()
    for _ in range(3):
        a.vcycle()
    saved = a.get_vars()
    path = str(tmp_path / "coupled.ckpt")
    a.checkpoint_save(path)
    ra = a.solve()
    b = Solver(case)
    b.set_inputs()
    b.checkpoint_load(path)
    for va, vb in zip(saved, b.get_vars()):
        for x, y in zip(va, vb):
            assert np.array_equal(x, y)
    rb = b.solve()
    assert ra["iters"] == rb["iters"]
    for va, vb in zip(a.get_vars(), b.get_vars()):
        for x, y in zip(va, vb):
            assert np.array_equal(x, y)
    # a one-variable checkpoint does not load into the two-variable solver
    one = Solver(W.lapse2d_bo(33, seed=6, levels=3, steps=8))
    one.set_inputs()
    p1 = str(tmp_path / "one.ckpt")
    one.checkpoint_save(p1)
    with pytest.raises(PgbError):
        b.checkpoint_load(p1)
    for s in (a, b, one):
        s.close()
