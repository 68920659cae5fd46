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
