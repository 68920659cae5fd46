"""Seeded synthetic elliptic problems on AMR hierarchies.

Every input the solver sees is generated here from a seed, so the GPU path,
the CPU checker and the benchmark all run on byte-identical arrays.

A hierarchy follows PAMR's conventions (include/pamr.h, src/gh.c):
vertex-centred grids, level ``L`` has spacing ``dx_1 / 2**(L-1)`` (refinement
ratio 2), a grid is given by its level and bounding box, and grid functions
are float64 arrays stored with x fastest (Fortran ``u(Nx,Ny,Nz)``; ``Nz=1`` in
2-D).

Workloads (names carry their sizes):

* ``poisson2d_<n>``: lap(u) = rho on [-1,1]^2, one n x n grid, u=0 on the
  boundary; rho is a sum of 8 Gaussians (amplitude U(-1,1), width
  U(0.05,0.15), centre U(-0.8,0.8)^2).
* ``conformal3d_<n>_<m>``: lap(psi) + 2 pi rho psi^5 = 0 on [-10,10]^3; base
  n^3 grid plus two nested 2:1 levels of m^3 boxes centred on the origin;
  psi = 1 on the boundary and as the initial guess; rho is a sum of 4
  Gaussians (amplitude U(0,0.005), width U(0.5,2), centre U(-0.5,0.5)^3).
  Amplitudes ten times larger give a compactness M/R of order one, where the
  equation has no regular solution and the reference FAS diverges; the
  coarsest MG grid is 9^3 (min_mg_cwidth 9) so that the Newton-Gauss-Seidel
  diagonal -6/dx^2 + 10 pi rho psi^4 stays negative there.
* ``poisson2d_uneven``: lap(u) = rho on [-1,1]^2, 129^2 base grid plus 4
  refined levels of 8-64 boxes each (odd sides drawn from [17,129], aligned
  to parent grid lines and clipped to the parent box); rho is a sum of 32
  Gaussians.
"""
from __future__ import annotations

import copy
import dataclasses
import math
from typing import List, Sequence, Tuple

import numpy as np

POISSON, CONFORMAL, LAPSE, NBS, COUPLED = 0, 1, 2, 3, 4
PDE_NAMES = {POISSON: "poisson", CONFORMAL: "conformal", LAPSE: "lapse", NBS: "nbs"}

# Operators that are not built into the library, as the level-operator
# expressions an application registers (pgb_operator_create): source count,
# L[u], dL/du. NBS is the Newtonian boson star's potential equation
# V_xx + V_yy + V_zz - (phi_r^2 + phi_i^2) = 0 (examples/nbs/num.f:85-246),
# sources phi_r and phi_i, in the hook's order of operations.
OPERATORS = {NBS: (2, "lap - (s0*s0 + s1*s1)", "j0")}
# operators of several elliptic variables solved together: (sources, one
# (L, dL/du) pair per variable); COUPLED is two variables u, w with
#   L_u = lap u - s0 (u - w) - s1,   L_w = lap w - s0 (w - u),
# s0 >= 0 coupling them (a negative semi-definite coupling, so the system
# stays definite), s1 the source
VAR_OPERATORS = {COUPLED: (2, (("lap - s0*(u - u1) - s1", "j0 - s0"), ("lap - s0*(u - u0)", "j0 - s0")))}

# transfer operators (values of PAMR's transfer bits, include/pamr.h:92-105)
STRAIGHT_INJECT, HW_RESTR, FW_RESTR = 1, 2, 3


class SplitMix64:
    """splitmix64 stream; ``uniform()`` returns doubles in [0,1) (53 bits)."""

    MASK = (1 << 64) - 1

    def __init__(self, seed: int):
        self.state = seed & self.MASK

    def next_u64(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & self.MASK
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & self.MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & self.MASK
        return z ^ (z >> 31)

    def uniform(self, lo: float = 0.0, hi: float = 1.0) -> float:
        return lo + (hi - lo) * ((self.next_u64() >> 11) * (1.0 / 9007199254740992.0))

    def randint(self, lo: int, hi: int) -> int:
        """uniform integer in [lo, hi]"""
        return lo + int(self.next_u64() % (hi - lo + 1))


@dataclasses.dataclass
class Grid:
    level: int                      # 1-based AMR level
    bbox: Tuple[float, ...]         # (x0,x1,y0,y1[,z0,z1])
    shape: Tuple[int, int, int]     # (Nx,Ny,Nz), Nz=1 in 2-D

    @property
    def size(self) -> int:
        return self.shape[0] * self.shape[1] * self.shape[2]

    def coords(self, d: int) -> np.ndarray:
        n = self.shape[d]
        lo, hi = self.bbox[2 * d], self.bbox[2 * d + 1]
        return lo + (hi - lo) / (n - 1) * np.arange(n)


@dataclasses.dataclass
class MGParams:
    """AMRD multigrid knobs (amrd/io.c:96-109 defaults, amrd/io.c:269-288)."""
    pre_swp: int = 2
    pst_swp: int = 2
    max_iter: int = 60
    min_iter: int = 1
    max_citer: int = 5000
    tol: float = 0.0          # absolute, on the finest-level residual norm
    crtol: float = 1.0e-3
    w0_r: float = 1.0
    w0_i: float = 1.0
    min_cwidth: int = 3
    interp_order: int = 2     # order used for the coarse-grid correction (mg_interp2)
    restr_u: int = HW_RESTR   # mg_hw_restr = [u rho], mg_fw_restr = [u_res]
    restr_res: int = FW_RESTR
    restr_src: int = HW_RESTR
    precision: int = 0        # 0: FP64 (bit-exact), 1: FP32 smoothing in FP64 defect correction


@dataclasses.dataclass
class Case:
    name: str
    pde: int
    dim: int
    base_shape: Tuple[int, int, int]
    base_bbox: Tuple[float, ...]
    grids: List[Grid]
    u0: List[np.ndarray]
    src: List[np.ndarray]
    params: MGParams
    # sources 1.. of operators with several (src_extra[k-1][i] = source k of grid i)
    src_extra: List[List[np.ndarray]] = dataclasses.field(default_factory=list)
    restr_src_extra: List[int] = dataclasses.field(default_factory=list)
    # coarsest AMR level of the MG hierarchy (solve_elliptics(L, ...), amrd/mg.c:20)
    min_level: int = 1
    # elliptic variables 1.. of operators with several (u_extra[v-1][i] = variable v of grid i)
    u_extra: List[List[np.ndarray]] = dataclasses.field(default_factory=list)

    @property
    def num_levels(self) -> int:
        return max(g.level for g in self.grids)

    @property
    def nsrc(self) -> int:
        if self.pde in VAR_OPERATORS:
            return VAR_OPERATORS[self.pde][0]
        return OPERATORS[self.pde][0] if self.pde in OPERATORS else 1

    @property
    def nvar(self) -> int:
        return len(VAR_OPERATORS[self.pde][1]) if self.pde in VAR_OPERATORS else 1

    def var(self, v: int) -> List[np.ndarray]:
        """initial values of elliptic variable v on every grid"""
        return self.u0 if v == 0 else self.u_extra[v - 1]

    def source(self, k: int) -> List[np.ndarray]:
        """source k of every grid"""
        return self.src if k == 0 else self.src_extra[k - 1]

    def restr_src_k(self, k: int) -> int:
        if k == 0:
            return self.params.restr_src
        return self.restr_src_extra[k - 1] if len(self.restr_src_extra) >= k else self.params.restr_src

    def level_dx(self, level: int) -> List[float]:
        return [(self.base_bbox[2 * d + 1] - self.base_bbox[2 * d]) / (self.base_shape[d] - 1)
                / 2 ** (level - 1) for d in range(self.dim)]

    def total_points(self) -> int:
        return sum(g.size for g in self.grids)


def _grid_from_bbox(level: int, bbox: Sequence[float], dx: Sequence[float], dim: int) -> Grid:
    shape = [1, 1, 1]
    for d in range(dim):
        shape[d] = int((bbox[2 * d + 1] - bbox[2 * d]) / dx[d] + 1.5)
    return Grid(level, tuple(float(b) for b in bbox), tuple(shape))


def _mesh(g: Grid, dim: int):
    """coordinate arrays broadcast to the (Nz,Ny,Nx) memory layout"""
    x = g.coords(0)[None, None, :]
    y = g.coords(1)[None, :, None]
    z = g.coords(2)[:, None, None] if dim == 3 else np.zeros((1, 1, 1))
    return x, y, z


def _gaussians(g: Grid, dim: int, blobs) -> np.ndarray:
    x, y, z = _mesh(g, dim)
    out = np.zeros((g.shape[2], g.shape[1], g.shape[0]))
    for (a, w, c) in blobs:
        r2 = (x - c[0]) ** 2 + (y - c[1]) ** 2
        if dim == 3:
            r2 = r2 + (z - c[2]) ** 2
        out = out + a * np.exp(-r2 / (w * w))
    return np.ascontiguousarray(out).reshape(-1)


def initial_residual_norm(case: Case) -> float:
    """max over finest-level grids of the RMS of L[u0] on interior points
    (the norm the V-cycle returns, amrd/util.c:73-103 with the hooks of
    examples/nbs/num.f:129-161, rhs = 0)."""
    lf = case.num_levels
    dx = case.level_dx(lf)
    best = 0.0
    for i, (g, u, s) in enumerate(zip(case.grids, case.u0, case.src)):
        if g.level != lf:
            continue
        v = u.reshape(g.shape[2], g.shape[1], g.shape[0])
        f = s.reshape(v.shape)
        f1 = case.src_extra[0][i].reshape(v.shape) if case.pde in (NBS, COUPLED) else None
        c = v[..., 1:-1, 1:-1] if case.dim == 2 else v[1:-1, 1:-1, 1:-1]
        if case.dim == 2:
            t = ((v[:, 1:-1, 2:] - 2 * c + v[:, 1:-1, :-2]) / (dx[0] * dx[0]) +
                 (v[:, 2:, 1:-1] - 2 * c + v[:, :-2, 1:-1]) / (dx[1] * dx[1]))
            fs = f[:, 1:-1, 1:-1]
            fs1 = f1[:, 1:-1, 1:-1] if f1 is not None else None
        else:
            t = ((v[1:-1, 1:-1, 2:] - 2 * c + v[1:-1, 1:-1, :-2]) / (dx[0] * dx[0]) +
                 (v[1:-1, 2:, 1:-1] - 2 * c + v[1:-1, :-2, 1:-1]) / (dx[1] * dx[1]) +
                 (v[2:, 1:-1, 1:-1] - 2 * c + v[:-2, 1:-1, 1:-1]) / (dx[2] * dx[2]))
            fs = f[1:-1, 1:-1, 1:-1]
            fs1 = f1[1:-1, 1:-1, 1:-1] if f1 is not None else None
        if case.pde == COUPLED:   # both variables' residuals in one norm
            w = case.u_extra[0][i].reshape(v.shape)
            cw = w[..., 1:-1, 1:-1] if case.dim == 2 else w[1:-1, 1:-1, 1:-1]
            if case.dim == 2:
                tw = ((w[:, 1:-1, 2:] - 2 * cw + w[:, 1:-1, :-2]) / (dx[0] * dx[0]) +
                      (w[:, 2:, 1:-1] - 2 * cw + w[:, :-2, 1:-1]) / (dx[1] * dx[1]))
            else:
                tw = ((w[1:-1, 1:-1, 2:] - 2 * cw + w[1:-1, 1:-1, :-2]) / (dx[0] * dx[0]) +
                      (w[1:-1, 2:, 1:-1] - 2 * cw + w[1:-1, :-2, 1:-1]) / (dx[1] * dx[1]) +
                      (w[2:, 1:-1, 1:-1] - 2 * cw + w[:-2, 1:-1, 1:-1]) / (dx[2] * dx[2]))
            ru = t - fs * (c - cw) - fs1
            rw = tw - fs * (cw - c)
            best = max(best, float(np.sqrt(np.mean(ru * ru + rw * rw))))
            continue
        if case.pde == POISSON:
            r = t - fs
        elif case.pde == NBS:
            r = t - (fs * fs + fs1 * fs1)
        elif case.pde == CONFORMAL:
            r = t + 2 * math.pi * fs * c ** 5
        else:
            r = t - fs * c
        best = max(best, float(np.sqrt(np.mean(r * r))))
    return best


def _finish(case: Case, rel_tol: float) -> Case:
    if rel_tol > 0:
        case.params.tol = rel_tol * initial_residual_norm(case)
    return case


def poisson2d(n: int = 129, seed: int = 0, rel_tol: float = 1e-10,
              params: MGParams | None = None) -> Case:
    rng = SplitMix64(0x5EED0001 + seed)
    blobs = []
    for _ in range(8):
        a = rng.uniform(-1, 1)
        w = rng.uniform(0.05, 0.15)
        c = (rng.uniform(-0.8, 0.8), rng.uniform(-0.8, 0.8))
        blobs.append((a, w, c))
    bbox = (-1.0, 1.0, -1.0, 1.0)
    g = Grid(1, bbox, (n, n, 1))
    case = Case(f"poisson2d_{n}", POISSON, 2, (n, n, 1), bbox, [g],
                [np.zeros(g.size)], [_gaussians(g, 2, blobs)], params or MGParams())
    return _finish(case, rel_tol)


def poisson3d_blobs(seed: int = 0):
    """the four Gaussians (amplitude, width, centre) of poisson3d"""
    rng = SplitMix64(0x5EED0005 + seed)
    blobs = []
    for _ in range(4):
        a = rng.uniform(0.0, 0.05)
        w = rng.uniform(0.5, 2.0)
        c = (rng.uniform(-0.5, 0.5), rng.uniform(-0.5, 0.5), rng.uniform(-0.5, 0.5))
        blobs.append((a, w, c))
    return blobs


def poisson3d_charge(blobs) -> float:
    """the integral of poisson3d's source over all space (each Gaussian
    a * exp(-r^2 / w^2) holds a * pi^(3/2) * w^3); the boundary cuts off a
    negligible tail"""
    return sum(a * math.pi ** 1.5 * w ** 3 for a, w, _ in blobs)


def poisson3d(n: int = 129, seed: int = 0, rel_tol: float = 1e-10,
              params: MGParams | None = None) -> Case:
    """the learned-initial-guess workload: lap u = rho on [-10,10]^3, one
    n^3 grid, u = 0 on the boundary, rho = 4 Gaussians drawn like
    conformal3d's source (amplitude U(0, 0.05): the linear equation has no
    existence limit)"""
    bbox = (-10.0, 10.0, -10.0, 10.0, -10.0, 10.0)
    g = Grid(1, bbox, (n, n, n))
    case = Case(f"poisson3d_{n}", POISSON, 3, (n, n, n), bbox, [g], [np.zeros(g.size)],
                [_gaussians(g, 3, poisson3d_blobs(seed))], params or MGParams())
    return _finish(case, rel_tol)


def conformal3d(n: int = 129, m: int = 65, seed: int = 0, rel_tol: float = 1e-10,
                params: MGParams | None = None, levels: int = 3) -> Case:
    rng = SplitMix64(0x5EED0002 + seed)
    blobs = []
    for _ in range(4):
        a = rng.uniform(0.0, 0.005)
        w = rng.uniform(0.5, 2.0)
        c = (rng.uniform(-0.5, 0.5), rng.uniform(-0.5, 0.5), rng.uniform(-0.5, 0.5))
        blobs.append((a, w, c))
    bbox = (-10.0, 10.0, -10.0, 10.0, -10.0, 10.0)
    dx1 = 20.0 / (n - 1)
    grids = [Grid(1, bbox, (n, n, n))]
    for lev in range(2, levels + 1):
        dx = dx1 / 2 ** (lev - 1)
        h = 0.5 * (m - 1) * dx
        grids.append(_grid_from_bbox(lev, (-h, h, -h, h, -h, h), [dx] * 3, 3))
    src = [_gaussians(g, 3, blobs) for g in grids]
    u0 = [np.ones(g.size) for g in grids]
    case = Case(f"conformal3d_{n}_{m}" + ("" if levels == 3 else f"_L{levels}"), CONFORMAL, 3,
                (n, n, n), bbox, grids, u0, src, params or MGParams(min_cwidth=9))
    return _finish(case, rel_tol)


def lapse_shell(seed: int = 0):
    """(radius, amplitude, width) of lapse2d_bo's Gaussian shell"""
    rng = SplitMix64(0x5EED0004 + seed)
    return rng.uniform(2.0, 6.0), rng.uniform(0.01, 0.1), rng.uniform(0.3, 1.0)


def shell_radius(r0: float, step: int, steps: int) -> float:
    """the shell breathes once over the run: R = r0 (1 + sin(2 pi step / steps) / 4)"""
    return r0 * (1.0 + 0.25 * math.sin(2.0 * math.pi * step / steps))


def lapse_source(g: Grid, radius: float, amp: float, width: float) -> np.ndarray:
    """S = amp exp(-((r - radius) / width)^2) on grid g (2-D)"""
    x, y, _ = _mesh(g, 2)
    r = np.sqrt(x * x + y * y)
    out = amp * np.exp(-((r - radius) / width) ** 2) * np.ones((1, g.shape[1], g.shape[0]))
    return np.ascontiguousarray(out).reshape(-1)


def lapse2d_bo_grids(n: int, seed: int, levels: int):
    """the fixed hierarchy of lapse2d_bo: the n^2 base grid on [-10,10]^2
    and one centred box per refined level (ratio 2), each covering the
    shell's whole excursion plus three widths, nested half a unit inside
    its parent, edges on the parent's grid lines"""
    r0, _, w = lapse_shell(seed)
    bbox = (-10.0, 10.0, -10.0, 10.0)
    dx1 = 20.0 / (n - 1)
    grids = [Grid(1, bbox, (n, n, 1))]
    half = min(9.0, 1.25 * r0 + 3.0 * w + 1.0)
    for lev in range(2, levels + 1):
        dxp = dx1 / 2 ** (lev - 2)
        h = dxp * math.floor(half / dxp)
        grids.append(_grid_from_bbox(lev, (-h, h, -h, h), [dxp / 2] * 2, 2))
        half = h - 0.5
    return bbox, grids


def lapse2d_bo(n: int = 257, seed: int = 0, levels: int = 4, step: int = 0, steps: int = 400,
               rel_tol: float = 1e-10, params: MGParams | None = None) -> Case:
    """one coarse step of the Berger-Oliger lapse sequence: the
    maximal-slicing lapse equation lap(alpha) = alpha S on the fixed
    hierarchy of lapse2d_bo_grids, alpha = 1 on the outer boundary (initial
    guess alpha = 1), S = the Gaussian shell at `step` of `steps` coarse
    steps (Courant 0.5: dt = dx/2 on the base grid; the shell's radius
    follows shell_radius). The tolerance is rel_tol times the initial
    residual of step 0, the same absolute tolerance for every step of the
    sequence, as AMRD keeps MG_tol fixed during a run."""
    r0, amp, w = lapse_shell(seed)
    bbox, grids = lapse2d_bo_grids(n, seed, levels)
    u0 = [np.ones(g.size) for g in grids]
    src0 = [lapse_source(g, shell_radius(r0, 0, steps), amp, w) for g in grids]
    case = Case(f"lapse2d_bo_{n}_L{levels}_s{seed}", LAPSE, 2, (n, n, 1), bbox, grids, u0, src0,
                params or MGParams())
    _finish(case, rel_tol)
    if step:
        case.src = [lapse_source(g, shell_radius(r0, step, steps), amp, w) for g in grids]
        case.name += f"_t{step}"
    return case


def poisson2d_uneven(seed: int = 0, n: int = 129, levels: int = 5, min_boxes: int = 8,
                     max_boxes: int = 64, min_side: int = 17, max_side: int = 129,
                     rel_tol: float = 1e-10, params: MGParams | None = None,
                     nblobs: int = 32) -> Case:
    rng = SplitMix64(0x5EED0003 + seed)
    blobs = []
    for _ in range(nblobs):
        a = rng.uniform(-1, 1)
        w = rng.uniform(0.05, 0.15)
        c = (rng.uniform(-0.8, 0.8), rng.uniform(-0.8, 0.8))
        blobs.append((a, w, c))
    bbox = (-1.0, 1.0, -1.0, 1.0)
    dx1 = 2.0 / (n - 1)
    grids = [Grid(1, bbox, (n, n, 1))]
    parents = [grids[0]]
    for lev in range(2, levels + 1):
        dxp = dx1 / 2 ** (lev - 2)
        dx = dxp / 2
        nb = rng.randint(min_boxes, max_boxes)
        mine = []
        while len(mine) < nb:
            p = parents[rng.randint(0, len(parents) - 1)]
            box = []
            ok = True
            for d in range(2):
                pn = p.shape[d]
                side = 2 * rng.randint((min_side - 1) // 2, (max_side - 1) // 2) + 1
                cells = (side - 1) // 2                   # parent cells covered
                p0 = rng.randint(0, max(0, pn - 2))
                p1 = min(pn - 1, p0 + cells)
                if p1 - p0 < 2:
                    ok = False
                    break
                lo = p.bbox[2 * d] + p0 * dxp
                hi = p.bbox[2 * d] + p1 * dxp
                box += [lo, hi]
            if not ok:
                continue
            mine.append(_grid_from_bbox(lev, box, [dx, dx], 2))
        grids += mine
        parents = mine
    src = [_gaussians(g, 2, blobs) for g in grids]
    u0 = [np.zeros(g.size) for g in grids]
    case = Case(f"poisson2d_uneven_s{seed}", POISSON, 2, (n, n, 1), bbox, grids, u0, src,
                params or MGParams())
    return _finish(case, rel_tol)


def _nbs_fields(g: Grid, dim: int, stars):
    """phi_r, phi_i of a few Gaussian boson-star profiles
    A exp(-r^2/w^2) (cos, sin)(k . x + phase) on grid g"""
    x, y, z = _mesh(g, dim)
    pr = np.zeros((g.shape[2], g.shape[1], g.shape[0]))
    pi_ = np.zeros_like(pr)
    for (a, w, c, kv, ph) in stars:
        r2 = (x - c[0]) ** 2 + (y - c[1]) ** 2
        arg = kv[0] * x + kv[1] * y + ph
        if dim == 3:
            r2 = r2 + (z - c[2]) ** 2
            arg = arg + kv[2] * z
        env = a * np.exp(-r2 / (w * w))
        pr = pr + env * np.cos(arg)
        pi_ = pi_ + env * np.sin(arg)
    return (np.ascontiguousarray(pr).reshape(-1), np.ascontiguousarray(pi_).reshape(-1))


def _nbs_stars(rng: SplitMix64, dim: int, count: int, half: float, wmin: float = 0.1, wmax: float = 0.25):
    stars = []
    for _ in range(count):
        a = rng.uniform(0.2, 1.0)
        w = rng.uniform(wmin, wmax) * half
        c = tuple(rng.uniform(-0.4, 0.4) * half for _ in range(dim))
        kv = tuple(rng.uniform(-2.0, 2.0) / w for _ in range(dim))
        stars.append((a, w, c, kv, rng.uniform(0, 2 * math.pi)))
    return stars


def nbs3d(n: int = 65, m: int = 33, seed: int = 0, levels: int = 2, rel_tol: float = 1e-10,
          params: MGParams | None = None) -> Case:
    """The Newtonian boson star's potential (examples/nbs): V_xx + V_yy + V_zz
    = phi_r^2 + phi_i^2 on [-1,1]^3, V = 0 on the boundary and as the initial
    guess; n^3 base grid plus nested 2:1 levels of m^3 boxes centred on the
    origin; phi = sum of 3 seeded Gaussian wave packets. Two sources, an
    operator the library does not build in: the application registers it as
    "lap - (s0*s0 + s1*s1)" (OPERATORS[NBS])."""
    rng = SplitMix64(0x5EED0006 + seed)
    stars = _nbs_stars(rng, 3, 3, 1.0)
    bbox = (-1.0, 1.0, -1.0, 1.0, -1.0, 1.0)
    dx1 = 2.0 / (n - 1)
    grids = [Grid(1, bbox, (n, n, n))]
    for lev in range(2, levels + 1):
        dx = dx1 / 2 ** (lev - 1)
        h = 0.5 * (m - 1) * dx
        grids.append(_grid_from_bbox(lev, (-h, h, -h, h, -h, h), [dx] * 3, 3))
    f = [_nbs_fields(g, 3, stars) for g in grids]
    case = Case(f"nbs3d_{n}_{m}" + ("" if levels == 2 else f"_L{levels}") + f"_s{seed}", NBS, 3,
                (n, n, n), bbox, grids, [np.zeros(g.size) for g in grids], [a for a, _ in f],
                params or MGParams(), src_extra=[[b for _, b in f]])
    return _finish(case, rel_tol)


def nbs2d_uneven(seed: int = 0, n: int = 65, levels: int = 3, min_boxes: int = 3,
                 max_boxes: int = 8, min_side: int = 9, max_side: int = 33,
                 rel_tol: float = 1e-10, params: MGParams | None = None) -> Case:
    """the nbs potential on an uneven 2-D hierarchy (poisson2d_uneven's box
    layout: odd sides aligned to parent lines and clipped to the parent),
    phi_r and phi_i as in nbs3d"""
    base = poisson2d_uneven(seed, n=n, levels=levels, min_boxes=min_boxes, max_boxes=max_boxes,
                            min_side=min_side, max_side=max_side, rel_tol=0, params=params, nblobs=1)
    rng = SplitMix64(0x5EED0007 + seed)
    stars = _nbs_stars(rng, 2, 6, 1.0, 0.25, 0.5)   # wide enough that every refined box sees them
    f = [_nbs_fields(g, 2, stars) for g in base.grids]
    case = Case(f"nbs2d_uneven_s{seed}", NBS, 2, base.base_shape, base.base_bbox, base.grids,
                [np.zeros(g.size) for g in base.grids], [a for a, _ in f], base.params,
                src_extra=[[b for _, b in f]])
    return _finish(case, rel_tol)


def _sub_grid(rng: SplitMix64, parent: Grid, level: int, dim: int, min_cells: int, max_cells: int) -> Grid:
    """a level-`level` grid inside `parent` (one level coarser), on its
    lattice: between min_cells and max_cells parent cells per side"""
    box = []
    dx = []
    for d in range(dim):
        pn = parent.shape[d]
        dxp = (parent.bbox[2 * d + 1] - parent.bbox[2 * d]) / (pn - 1)
        cells = rng.randint(min_cells, max(min_cells, min(max_cells, pn - 1)))
        p0 = rng.randint(0, pn - 1 - cells)
        box += [parent.bbox[2 * d] + p0 * dxp, parent.bbox[2 * d] + (p0 + cells) * dxp]
        dx.append(dxp / 2)
    return _grid_from_bbox(level, box, dx, dim)


def regrid_pair(seed: int = 0, dim: int = 2, n: int = 33, finer: bool = False):
    """an AMR hierarchy and the one a regrid replaces it with, as PAMR's
    compose_hierarchy sees them (levels 2.. recomposed, the base grid kept).
    Old: level 2 grids A, B, C (B may overlap A), level 3 grids in A and B.
    New: level 2 keeps A and C and adds D; level 3 keeps the old grid in A
    and adds two inside A (overlapping it or not); with finer, a new level 4
    inside the kept level-3 grid. Every new grid of level L lies inside an
    old grid of level L-1, so the interpolation reaches all its points, and
    inside a new grid of level L-1 (proper nesting). Old u and sources are
    seeded random numbers (``regrid_data``); new ones start at zero."""
    rng = SplitMix64(0x5EED0007 + seed)
    bbox = (-1.0, 1.0, -1.0, 1.0, -1.0, 1.0)[:2 * dim]
    shape = (n, n, n if dim == 3 else 1)
    base = Grid(1, bbox, shape)
    lo, hi = (3, (n - 1) // 2) if dim == 2 else (2, (n - 1) // 2)
    a, b, c = (_sub_grid(rng, base, 2, dim, lo, hi) for _ in range(3))
    a3 = _sub_grid(rng, a, 3, dim, lo, hi)
    b3 = _sub_grid(rng, b, 3, dim, lo, hi)
    old = [base, a, b, c, a3, b3]
    d = _sub_grid(rng, base, 2, dim, lo, hi)
    new = [base, a, c, d, a3] + [_sub_grid(rng, a, 3, dim, lo, hi) for _ in range(2)]
    if finer:
        new.append(_sub_grid(rng, a3, 4, dim, 2, hi))
    prm = MGParams()
    mk = lambda name, grids: Case(name, POISSON, dim, shape, bbox, grids,
                                  [np.zeros(g.size) for g in grids], [np.zeros(g.size) for g in grids], prm)
    tag = f"regrid{dim}d_{n}_s{seed}" + ("_L4" if finer else "")
    return mk(tag + "_old", old), mk(tag + "_new", new)


def regrid_data(case: Case, seed: int) -> Case:
    """seeded random u and source on every grid of `case` (in place)"""
    rng = np.random.default_rng(seed)
    case.u0 = [rng.standard_normal(g.size) for g in case.grids]
    case.src = [rng.standard_normal(g.size) for g in case.grids]
    return case


def coupled_from(base: Case, seed: int = 0, rel_tol: float = 1e-10) -> Case:
    """the coupled two-variable system (VAR_OPERATORS[COUPLED]) on the grids
    of `base`: coupling s0 = 1 + three seeded Gaussians of amplitude U(0, 4),
    source s1 = four seeded Gaussians of amplitude U(-1, 1), widths U(0.1, 0.3)
    of the domain half-width; both variables start at 0"""
    rng = SplitMix64(0x5EED0008 + seed)
    half = 0.5 * (base.base_bbox[1] - base.base_bbox[0])
    cen = [0.5 * (base.base_bbox[2 * d] + base.base_bbox[2 * d + 1]) for d in range(base.dim)]

    def blobs(n, lo, hi):
        out = []
        for _ in range(n):
            a = rng.uniform(lo, hi)
            w = rng.uniform(0.1, 0.3) * half
            c = tuple(cen[d] + rng.uniform(-0.5, 0.5) * half for d in range(base.dim)) + (0.0,) * (3 - base.dim)
            out.append((a, w, c))
        return out
    b0, b1 = blobs(3, 0.0, 4.0), blobs(4, -1.0, 1.0)
    grids = base.grids
    s0 = [1.0 + _gaussians(g, base.dim, b0) for g in grids]
    s1 = [_gaussians(g, base.dim, b1) for g in grids]
    case = Case(f"coupled_{base.name}", COUPLED, base.dim, base.base_shape, base.base_bbox, grids,
                [np.zeros(g.size) for g in grids], s0, copy.deepcopy(base.params),
                src_extra=[s1], u_extra=[[np.zeros(g.size) for g in grids]], min_level=base.min_level)
    return _finish(case, rel_tol)


def with_min_level(case: Case, level: int) -> Case:
    """the case solved on the MG hierarchy built from AMR level `level` up
    (solve_elliptics(level, ...), amrd/mg.c:20; level = the finest is the
    hierarchy of the V-cycle inside the evolution iteration,
    amrd/evolve.c:454); grids below it keep their values"""
    case.min_level = level
    case.name += f"_min{level}"
    return case

