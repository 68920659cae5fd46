"""The device Berger-Oliger bookkeeping (pgb_bo.cu) against the oracle's
restatement of amrd/evolve.c, bit for bit, on random data: both
extrapolation methods at times whose coefficients round, the update of the
extrapolation levels over a three-level hierarchy of grids of different
sizes (L1 = 1 and L1 > 1, with and without the eps_c correction), and the
brs copy."""
import ctypes as C

import numpy as np
import pytest

from oracle import portrun

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
D = C.POINTER(C.c_double)


@pytest.fixture(scope="module")
def olib():
    L = C.CDLL(portrun.build())
    L.oracle_mg_extrap.argtypes = [C.c_int] + [C.c_double] * 4 + [D] * 4 + [C.c_long]
    L.oracle_update_mg_extrap_vars.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int), C.c_int,
                                               C.POINTER(C.c_int), C.POINTER(D), C.POINTER(D),
                                               C.POINTER(D), C.POINTER(D), C.POINTER(C.c_long), C.c_double]
    L.oracle_set_mg_brs_vars.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(D),
                                         C.POINTER(D), C.POINTER(C.c_long)]
    return L


def _p(a):
    return a.ctypes.data_as(D)


def _pp(arrs):
    return (D * len(arrs))(*[_p(a) for a in arrs])


def _dev(a):
    return torch.from_numpy(a.copy()).cuda()


@pytest.mark.parametrize("method", [0, 1])
@pytest.mark.parametrize("times", [(0.7, 0.9, 0.1, 0.3), (1.0 / 3, 0.5, 1.0 / 7, 0.2)])
def test_extrap_matches_oracle(olib, method, times):
    from pamr_amrd_gb300 import bo
    rng = np.random.default_rng(method * 10 + int(times[0] * 100))
    n = 100003
    m1, e1, e2 = (rng.standard_normal(n) for _ in range(3))
    want = np.zeros(n)
    assert olib.oracle_mg_extrap(method, *times, _p(want), _p(m1), _p(e1), _p(e2), n) == 0
    d0 = torch.zeros(n, dtype=torch.float64, device="cuda")
    dm1, de1, de2 = _dev(m1), _dev(e1), _dev(e2)
    bo.mg_extrap(method, *times, d0.data_ptr(), dm1.data_ptr(), de1.data_ptr(), de2.data_ptr(), n)
    torch.cuda.synchronize()
    assert np.array_equal(d0.cpu().numpy(), want)


@pytest.mark.parametrize("L1,eps_c", [(1, 1.0), (2, 1.0), (1, 0.0), (1, 0.3)])
def test_update_and_brs_match_oracle(olib, L1, eps_c):
    from pamr_amrd_gb300 import bo
    rng = np.random.default_rng(L1 * 7 + int(eps_c * 10))
    levels = [1, 2, 2, 3]
    sizes = [4097, 1000, 333, 2049]
    rho_tm = [2, 2, 4, 2]
    e1, e2, m1, brs = ([rng.standard_normal(s) for s in sizes] for _ in range(4))
    de1, de2, dm1, dbrs = ([_dev(a) for a in arrs] for arrs in (e1, e2, m1, brs))
    # device first (the oracle updates its arrays in place)
    bo.set_mg_brs_vars(2, 3, levels, [t.data_ptr() for t in dbrs], [t.data_ptr() for t in dm1], sizes)
    bo.update_mg_extrap_vars(L1, 3, rho_tm, levels, [t.data_ptr() for t in de1], [t.data_ptr() for t in de2],
                             [t.data_ptr() for t in dm1], [t.data_ptr() for t in dbrs], sizes, eps_c)
    torch.cuda.synchronize()
    g = len(levels)
    olib.oracle_set_mg_brs_vars(2, 3, g, (C.c_int * g)(*levels), _pp(brs), _pp(m1), (C.c_long * g)(*sizes))
    olib.oracle_update_mg_extrap_vars(L1, 3, (C.c_int * 4)(*rho_tm), g, (C.c_int * g)(*levels), _pp(e1), _pp(e2),
                                      _pp(m1), _pp(brs), (C.c_long * g)(*sizes), eps_c)
    for k in range(g):
        assert np.array_equal(dbrs[k].cpu().numpy(), brs[k])
        assert np.array_equal(de1[k].cpu().numpy(), e1[k])
        assert np.array_equal(de2[k].cpu().numpy(), e2[k])
