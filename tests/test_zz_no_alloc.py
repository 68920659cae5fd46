"""pgb_residual_norm_noalloc -- the residual-and-norm entry point for callers
that cannot allocate device memory (applications that budget all device
memory themselves, or that must not let an allocation synchronize the device
between their own launches) -- checked through the C ABI: its norm against
the residual the ordinary solver entry point (pgb_vcycle) reports, and, on a
grid with an AMR-boundary mask, its res array against the CPU checker's
residual hook (oracle/mg_ops.c, the pattern of examples/nbs/num.f:129-161)
at every cmask-ON point, with the OFF points left untouched; each on two
calls in a row. This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from oracle import portrun
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


def _noalloc(pde, dim, shape, dx, u, src, rhs=None, mask=None, res0=None):
    """res and norm from the entry point (mask: uint8, 1 = CMASK_ON)"""
    f = _bind()
    sh = (C.c_int * 3)(*shape)
    dxa = (C.c_double * 3)(*(list(dx) + [1.0] * (3 - len(dx))))
    d_u = torch.from_numpy(np.ascontiguousarray(u)).cuda()
    d_src = torch.from_numpy(np.ascontiguousarray(src)).cuda()
    d_rhs = torch.from_numpy(np.ascontiguousarray(rhs)).cuda() if rhs is not None else torch.zeros_like(d_u)
    d_res = torch.from_numpy(np.ascontiguousarray(res0)).cuda() if res0 is not None else torch.zeros_like(d_u)
    d_mask = torch.from_numpy(np.ascontiguousarray(mask, dtype=np.uint8)).cuda() if mask is not None else None
    d_norm = torch.zeros(1, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = f(pde, dim, sh, dxa, d_u.data_ptr(), d_rhs.data_ptr(), d_src.data_ptr(),
           d_mask.data_ptr() if d_mask is not None else None, d_res.data_ptr(), d_norm.data_ptr(), None)
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
    g = case.grids[0]
    dx = [(g.bbox[2 * d + 1] - g.bbox[2 * d]) / (g.shape[d] - 1) for d in range(case.dim)]
    for _ in range(2):          # two calls in a row, each against a fresh V-cycle
        want = s.vcycle()       # finest residual reported by the ordinary entry point
        u = s.get_u()[0]
        got, res = _noalloc(case.pde, case.dim, g.shape, dx, u, case.src[0])
        assert abs(got - want) <= RTOL * want
        assert np.isfinite(res).all()
    s.close()


def _oracle_residual(pde, dim, shape, dx, u, src, rhs, mask):
    """the checker's residual hook: res at ON points and the RMS norm"""
    lib_o = C.CDLL(portrun.build())

    class OG(C.Structure):
        _fields_ = [("dim", C.c_int), ("shape", C.c_int * 3), ("dx", C.c_double * 3)]

    f = lib_o.oracle_residual
    dp = C.POINTER(C.c_double)
    f.argtypes = [C.c_int, C.POINTER(OG), dp, dp, dp, C.POINTER(dp), dp]
    f.restype = C.c_double
    og = OG(dim, (C.c_int * 3)(*shape), (C.c_double * 3)(*(list(dx) + [1.0] * (3 - len(dx)))))
    res = np.zeros_like(u)
    srcs = [np.ascontiguousarray(src)]
    sp = (dp * 1)(*[a.ctypes.data_as(dp) for a in srcs])
    m = np.ascontiguousarray(mask, dtype=np.float64)
    norm = f(pde, C.byref(og), res.ctypes.data_as(dp), np.ascontiguousarray(rhs).ctypes.data_as(dp),
             np.ascontiguousarray(u).ctypes.data_as(dp), sp, m.ctypes.data_as(dp))
    return norm, res


@pytest.mark.parametrize("make,level,pde", [
    (lambda: W.poisson2d_uneven(seed=3, n=65, levels=3, min_boxes=2, max_boxes=4, min_side=17, max_side=33),
     3, W.POISSON),
    (lambda: W.conformal3d(33, 17, seed=2), 3, W.CONFORMAL)], ids=["uneven2d_finest", "conformal3d_finest"])
def test_noalloc_masked_residual_matches_oracle_twice(make, level, pde):
    """a finest box of a multi-box hierarchy with its boundary cmask (OFF on
    its AMR boundaries) converted to uint8, 1 = CMASK_ON: res at the ON
    points equals the checker's residual bit for bit, the OFF points keep
    what the array held, and the norm agrees to summation order"""
    case = make()
    hs = Solver(case, host_only=True)
    L = hs.num_levels()
    info = hs.box_info(L, 0)
    shape = info["shape"]
    mask = hs.cmask(L, 0, "bdy")                 # 1.0 / 0.0 as PAMR stores it
    hs.close()
    dim = case.dim
    dx = [(info["bbox"][2 * d + 1] - info["bbox"][2 * d]) / (shape[d] - 1) for d in range(dim)]
    n = shape[0] * shape[1] * shape[2]
    rng = np.random.default_rng(11)
    assert 0 < mask.sum() < n
    for call in range(2):                        # two calls in a row, different data
        u = 1.0 + 0.1 * rng.standard_normal(n)
        src = 0.01 * rng.random(n)
        rhs = rng.standard_normal(n)
        sentinel = np.full(n, 7.25 + call)
        got, res = _noalloc(pde, dim, shape, dx, u, src, rhs, (mask != 0).astype(np.uint8), sentinel)
        want, res_o = _oracle_residual(pde, dim, shape, dx, u, src, rhs, mask)
        on = mask != 0
        interior = np.zeros(shape[::-1], dtype=bool)
        if dim == 2:
            interior[:, 1:-1, 1:-1] = True
        else:
            interior[1:-1, 1:-1, 1:-1] = True
        interior = interior.reshape(-1)
        sel = on & interior                      # the hook works on interior ON points
        assert np.array_equal(res[sel], res_o[sel])
        assert np.array_equal(res[~sel], sentinel[~sel])
        assert abs(got - want) <= RTOL * want


def test_noalloc_empty_mask_gives_nan_like_the_hook():
    """no ON point: the RMS divides 0 by 0, NaN, as the reference's hook does
    (examples/nbs/num.f:158)"""
    shape = (17, 17, 1)
    n = 17 * 17
    got, res = _noalloc(W.POISSON, 2, shape, [0.125, 0.125], np.zeros(n), np.zeros(n), mask=np.zeros(n, np.uint8),
                        res0=np.zeros(n))
    assert np.isnan(got)
    assert not res.any()


def test_noalloc_rejects_grids_beyond_its_scratch():
    f = _bind()
    shape = (C.c_int * 3)(2049, 2049, 1)     # 65 x 257 tiles > 4095
    dx = (C.c_double * 3)(1.0, 1.0, 1.0)
    rc = f(0, 2, shape, dx, None, None, None, None, None, None, None)
    assert rc == 2
