"""Host-side pieces of bench.py: the algorithmic-bytes model of a V-cycle
(the numerator of the whole-solve roofline) on a host-only hierarchy."""
import bench
from pamr_amrd_gb300 import workloads as W
from pamr_amrd_gb300.solver import Solver


def test_vcycle_bytes_single_grid_hierarchy():
    # one 17^3 grid: MG levels 3^3, 5^3, 9^3, 17^3 with 1, 27, 343, 3375 interior points
    s = Solver(W.poisson3d(17, seed=0), host_only=True)
    mb = bench.solve_model_bytes(s, 2, 2, 16.0)
    s.close()
    assert mb["interior_points"] == [1, 27, 343, 3375]
    # (27 + 343 + 3375) x (4 x 16 + 32 + 24 + 40 + 24) + 24 x ((27+1) + (343+27) + (3375+343))
    assert mb["bytes_per_cycle"] == 787864.0
    assert mb["coarsest_point_sweep_bytes"] == 16.0


def test_vcycle_bytes_count_every_box_of_a_level():
    case = W.poisson2d_uneven(seed=1)
    s = Solver(case, host_only=True)
    mb = bench.solve_model_bytes(s, 2, 2, 32.0)
    n = mb["interior_points"]
    assert len(n) == s.num_levels()
    for L in range(1, s.num_levels() + 1):
        tot = 0
        for b in range(s.level_nbox(L)):
            nx, ny, _ = s.box_info(L, b)["shape"]
            tot += (nx - 2) * (ny - 2)
        assert n[L - 1] == tot
    s.close()
