"""The guess policy (host logic, no GPU): it starts with one plain solve,
keeps guessing while guessed solves need fewer V-cycles and less time than
the plain one, and goes back to the plain initial guess after `patience`
strikes in a row."""
from pamr_amrd_gb300.learned import GuessPolicy


def test_first_solve_is_plain():
    p = GuessPolicy()
    assert not p.use_guess()
    p.record(11, False, 25.0)
    assert p.use_guess()


def test_guess_that_pays_stays_on():
    p = GuessPolicy()
    p.record(11, False, 25.0)
    for _ in range(5):
        p.record(10, True, 24.2)
    assert p.use_guess()


def test_no_fewer_cycles_turns_it_off():
    p = GuessPolicy(patience=2)
    p.record(11, False, 25.0)
    p.record(11, True, 24.0)
    assert p.use_guess()
    p.record(12, True, 24.0)
    assert not p.use_guess()


def test_fewer_cycles_but_slower_turns_it_off():
    p = GuessPolicy(patience=2)
    p.record(11, False, 7.7)
    p.record(10, True, 8.4)
    p.record(10, True, 8.4)
    assert not p.use_guess()


def test_a_good_solve_resets_the_strikes():
    p = GuessPolicy(patience=2)
    p.record(11, False, 25.0)
    p.record(11, True, 25.0)
    p.record(10, True, 24.0)
    p.record(11, True, 25.0)
    assert p.use_guess()
