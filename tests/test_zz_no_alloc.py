"""pgb_residual_norm_noalloc -- the residual-and-norm entry point for callers
that cannot allocate device memory (applications that budget all device
memory themselves, or that must not let an allocation synchronize the device
between their own launches) -- checked through the C ABI against the
residual the ordinary solver entry point (pgb_vcycle) reports, on two calls
in a row, and for its size limit. This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from pamr_amrd_gb300 import workloads as W
from pamr_amrd_gb300.solver import Solver, lib

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

RTOL = 1e-12   # the tolerance the FP64 parity tests use for norms


def _bind():
    L = lib()
    f = L.pgb_residual_norm_noalloc
    f.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double), C.c_void_p,
                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


def _noalloc_norm(case, u, src):
    f = _bind()
    g = case.grids[0]
    shape = (C.c_int * 3)(*g.shape)
    dx = (C.c_double * 3)(*[(g.bbox[2 * d + 1] - g.bbox[2 * d]) / (g.shape[d] - 1)
                            for d in range(case.dim)] + [1.0] * (3 - case.dim))
    d_u = torch.from_numpy(np.ascontiguousarray(u)).cuda()
    d_src = torch.from_numpy(np.ascontiguousarray(src)).cuda()
    d_rhs = torch.zeros_like(d_u)
    d_res = torch.zeros_like(d_u)
    d_norm = torch.zeros(1, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = f(case.pde, case.dim, shape, dx, d_u.data_ptr(), d_rhs.data_ptr(), d_src.data_ptr(),
           None, d_res.data_ptr(), d_norm.data_ptr(), None)
    torch.cuda.synchronize()
    assert rc == 0
    return float(d_norm.item()), d_res.cpu().numpy()


@pytest.mark.parametrize("make", [lambda: W.poisson2d(129, seed=4),
                                  lambda: W.conformal3d(33, 17, seed=1, levels=1)],
                         ids=["poisson2d_129", "conformal3d_33"])
def test_noalloc_residual_matches_vcycle_twice(make):
    case = make()
    s = Solver(case)
    s.set_inputs()
    s.prepare()
    for _ in range(2):          # two calls in a row, each against a fresh V-cycle
        want = s.vcycle()       # finest residual reported by the ordinary entry point
        u = s.get_u()[0]
        got, res = _noalloc_norm(case, u, case.src[0])
        assert abs(got - want) <= RTOL * want
        assert np.isfinite(res).all()
    s.close()


def test_noalloc_rejects_grids_beyond_its_scratch():
    f = _bind()
    shape = (C.c_int * 3)(2049, 2049, 1)     # 65 x 257 tiles > 4095
    dx = (C.c_double * 3)(1.0, 1.0, 1.0)
    rc = f(0, 2, shape, dx, None, None, None, None, None, None, None)
    assert rc == 2
