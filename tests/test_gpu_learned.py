"""The learned initial guess in a solve (GPU): a net trained briefly on
multigrid-generated pairs of the poisson3d workload guesses u, and the
plain multigrid then runs to tolerance from that guess. Whatever the
guess's quality, the solve converges and lands on the same discrete
solution as the solve from u = 0."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.mark.parametrize("precision", [0, 1])
def test_guessed_solve_converges_to_the_plain_solution(precision):
    from pamr_amrd_gb300 import learned as Lm
    from pamr_amrd_gb300 import workloads as W
    from pamr_amrd_gb300.solver import Solver
    n = 65
    h = 20.0 / (n - 1)
    blobs, U = Lm.make_dataset(n, range(16), torch)
    model = Lm.Scaled(Lm.Net(n, seed=4), Lm.fit_gain(n, blobs, U, torch), h)
    losses = Lm.train(model, blobs, U, torch, epochs=2, lr=1e-3)
    assert np.isfinite(losses).all()
    case = W.poisson3d(n, seed=100000)
    case.params.precision = precision
    sv = Solver(case)
    rho = Lm.rho_on_device(n, W.poisson3d_blobs(100000), torch)
    zero = torch.zeros(n ** 3, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()   # the solver copies on its own stream
    sv.set_inputs_device([zero.data_ptr()], [rho.data_ptr()])
    r0 = sv.solve()
    u0 = np.concatenate(sv.get_u())
    guess = torch.zeros_like(zero)
    model.predict(rho, guess, sv.stream())
    sv.set_inputs_device([guess.data_ptr()], [rho.data_ptr()])
    r1 = sv.solve()
    u1 = np.concatenate(sv.get_u())
    g = guess.cpu().numpy().reshape(n, n, n)
    assert np.isfinite(g).all() and not np.any(g[0]) and not np.any(g[:, :, -1])
    assert r0["res_final"] <= case.params.tol and r1["res_final"] <= case.params.tol
    assert np.abs(u1 - u0).max() <= 1e-8 * np.abs(u0).max()
    sv.close()
    model.net.close()


def _trained(n, pairs, epochs, torch):
    from pamr_amrd_gb300 import learned as Lm
    h = 20.0 / (n - 1)
    blobs, U = Lm.make_dataset(n, range(pairs), torch)
    model = Lm.Scaled(Lm.Net(n, seed=4), Lm.fit_gain(n, blobs, U, torch), h)
    Lm.train(model, blobs, U, torch, epochs=epochs, lr=1e-3)
    return model


def test_corrupt_guess_falls_back_to_the_plain_solve():
    """a guess with a NaN in it (a corrupt prediction, injected from the
    host) is replaced on the device by u = 0: the solve is the plain solve,
    cycle for cycle and bit for bit, and the rejection is counted"""
    from pamr_amrd_gb300 import learned as Lm
    from pamr_amrd_gb300 import workloads as W
    from pamr_amrd_gb300.solver import Solver
    n = 65
    h = 20.0 / (n - 1)
    model = Lm.Scaled(Lm.Net(n, seed=5), 1.0, h)    # untrained: any guess will do
    case = W.poisson3d(n, seed=100001)
    sv = Solver(case)
    rho = Lm.rho_on_device(n, W.poisson3d_blobs(100001), torch)
    zero = torch.zeros(n ** 3, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    sv.set_inputs_device([zero.data_ptr()], [rho.data_ptr()])
    r0 = sv.solve()
    u0 = np.concatenate(sv.get_u())
    guess = torch.zeros_like(zero)
    model.predict(rho, guess, sv.stream(), rescale=False)
    torch.cuda.synchronize()
    guess[n * n * (n // 2) + n * (n // 2) + n // 2] = float("nan")
    before = model.net.rejected_guesses()
    model.net.rescale(rho.data_ptr(), guess.data_ptr(), h, sv.stream())
    sv.set_inputs_device([guess.data_ptr()], [rho.data_ptr()])
    r1 = sv.solve()
    u1 = np.concatenate(sv.get_u())
    assert model.net.rejected_guesses() == before + 1
    assert not torch.any(guess != 0)
    assert r1["iters"] == r0["iters"]
    assert np.array_equal(u1, u0)
    sv.close()
    model.net.close()


def test_trained_net_cuts_vcycles_on_held_out_sources():
    """the gain: a net trained on multigrid-generated pairs, guessing u for
    sources it has not seen, takes fewer V-cycles on average than the plain
    solve from u = 0 (mixed form, same tolerance)"""
    from pamr_amrd_gb300 import learned as Lm
    from pamr_amrd_gb300 import workloads as W
    from pamr_amrd_gb300.solver import Solver
    n = 65
    model = _trained(n, 128, 6, torch)
    plain, guessed = [], []
    for seed in range(200000, 200006):
        case = W.poisson3d(n, seed=seed)
        case.params.precision = 1
        sv = Solver(case)
        rho = Lm.rho_on_device(n, W.poisson3d_blobs(seed), torch)
        zero = torch.zeros(n ** 3, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        sv.set_inputs_device([zero.data_ptr()], [rho.data_ptr()])
        plain.append(sv.solve()["iters"])
        guess = torch.zeros_like(zero)
        model.predict(rho, guess, sv.stream())
        sv.set_inputs_device([guess.data_ptr()], [rho.data_ptr()])
        r = sv.solve()
        assert r["res_final"] <= case.params.tol
        guessed.append(r["iters"])
        sv.close()
    assert np.mean(guessed) < np.mean(plain), (guessed, plain)
    model.net.close()
