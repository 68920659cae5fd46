/*
 * Mixed-precision kernels of libpamr_gb300 (sm_103a): FP32 smoothing and
 * FP32 prolongation inside FP64 defect correction.
 *
 * Every smoothing block of the FAS V-cycle (MG_pre_swp / MG_pst_swp sweeps,
 * amrd/mg.c:135-141, 161-167) works on a correction E in FP32:
 *     D = rhs - L[u]   (FP64, stored in FP32)     C = dL/du - lap part (FP32)
 *     red-black Gauss-Seidel on  lap E + C E = D  (FP32)
 *     u = u + E        (FP64)
 * D comes from FP64 passes the V-cycle runs anyway:
 *   - down sweep, level below the finest: the FAS right-hand-side pass
 *     (k_fas_defect) evaluates L[u] once for both rhs and D;
 *   - the residual pass after pre-smoothing (k_residual_fast) leaves
 *     D = -res for the post-smoothing block of the same level, and on the
 *     finest level for the next cycle's pre-smoothing block.
 * The coarse-grid correction (f - lop)/w0 is formed in FP64, stored once in
 * FP32 (X), interpolated in FP32 and becomes the starting value of E for the
 * post-smoothing block, so L[u + E] = rhs is solved from the pre-smoothing
 * residual with no further FP64 pass. Points the smoother never relaxes
 * (box boundaries, cmask-off points) take the FP64-interpolated correction
 * instead, so values that only change through corrections never collect
 * FP32 rounding. The V-cycle keeps every FP64 piece of the reference:
 * residuals, restriction, FAS right-hand sides, coarsest-grid solve and the
 * finest-level norm; for the nonlinear conformal operator the FP32 sweeps are
 * the linearised (Newton) sweeps and the next FP64 residual sees what the
 * linearisation left out.
 *
 * FP64 on this part runs at 2 operations per clock per SM (FP32: 128), so
 * the FP64 passes here are written for the fewest FP64 instructions: fused
 * multiply-adds, products with 1/dx^2, and FP32 wherever the value only
 * steers the smoother. Nothing here is compared bit for bit.
 */
#include <cuda.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "pgb_dev.h"
#include "pgb_opgrid.cuh"
#include "pgb_op.cuh"
#include "pgb_weights.cuh"

static __thread char g_err32[256];
static unsigned long long g_launches32 = 0;

extern "C" unsigned long long pgb_dev_launches32(void) { return g_launches32; }

static int check32(const char *what)
{
   g_launches32++;
   cudaError_t e = cudaGetLastError();
   if (e != cudaSuccess) {
      snprintf(g_err32, sizeof(g_err32), "%s: %s", what, cudaGetErrorString(e));
      return 1;
   }
   return 0;
}

extern "C" const char *pgb_dev_error32(void) { return g_err32; }

/* the small-level kernel's program being recorded (per host thread), 0 when
 * not recording (pgb_dev.h, pgb_tail_begin) */
static __thread pgb_tail_prog *g_tp = 0;
static __thread int g_tp_bad = 0, g_tp_solo = 0;

/* a pass the small-level kernel does not run: recording fails */
static int tail_refuse(void)
{
   g_tp_bad = 2;
   return 1;
}

#define NT (PGB_TX * PGB_TY)

/* Pointers a kernel body reads or writes through: restrict-qualified in the
 * standalone kernels, plain in the small-level kernel (k_tail), where one
 * step writes what another step of the same launch reads, so the loads must
 * stay on the coherent path. */
template <bool TAIL, class X> struct rp {
   typedef X *__restrict__ t;
};
template <class X> struct rp<true, X> {
   typedef X *t;
};
#define RP(X) typename rp<TAIL, X>::t

/* launches the instantiation of an operator kernel for the level
 * operator's form: compiled built-in (PROG = false) or program (true) */
#define OPLAUNCH(kern, pde, grid, blk, smem, st, ...)                                   \
   do {                                                                                 \
      if ((pde) == PGB_OPK_PROGRAM) kern<true><<<(grid), (blk), (smem), (st)>>>(__VA_ARGS__); \
      else kern<false><<<(grid), (blk), (smem), (st)>>>(__VA_ARGS__);                   \
   } while (0)
#define TWO_PI 6.283185307179586

/* the FP32 arrays of a box: correction, defect, Jacobian term, coarse correction */
enum { W_E = PGB_W32_E, W_D = 1, W_C = 2, W_X = 3, W_E2 = PGB_W32_E2 };

/* the correction array of slot sl (W_E or W_E2), selected without indexing
 * a register copy of the box by a runtime value (which would move the copy
 * to local memory) */
__device__ __forceinline__ float *eslot(const pgb_dbox &b, int sl)
{
   return sl == W_E2 ? b.w32[W_E2] : b.w32[W_E];
}

/* index into a box's FP32 arrays (rows padded to the pitch wy) */
__device__ __forceinline__ long wq(const pgb_dbox &b, int i, int j, int k)
{
   return i + (long)b.wy * j + b.wz * k;
}

__device__ __forceinline__ bool interior32(const pgb_dbox &b, int i, int j, int k, int dim)
{
   return i >= 1 && i <= b.n[0] - 2 && j >= 1 && j <= b.n[1] - 2 &&
          (dim == 2 ? k == 0 : (k >= 1 && k <= b.n[2] - 2));
}

/* the points relax visits: interior and cmask_bdy ON (num.f:211-232) */
__device__ __forceinline__ bool relaxed32(const pgb_dbox &b, int i, int j, int k, long p, int dim)
{
   return interior32(b, i, j, k, dim) && ((b.flags & PGB_BOX_BDY_INTERIOR) || b.cmask_bdy[p]);
}

/* Plane split of a level's tiles: a kernel over lv.ntiles x split CTAs
 * gives CTA b the planes [k0, k0 + nk) of tile b / split (split divides
 * the tile depth; bx is the CTA's index, blockIdx.x in a standalone launch).
 * Levels with few tiles (a 65^3 box in tiles of 8 planes
 * is 243 CTAs for 152 SMs) get enough CTAs to hide load latency. */
struct tile_part {
   pgb_tile tl;
   int kk0, nk;   /* first plane within the tile, planes */
};

__device__ __forceinline__ tile_part tile_split(const pgb_tile *tiles, const pgb_dlevel &lv, int split, int bx)
{
   tile_part t;
   t.tl = tiles[bx / split];
   const int kz = lv.dim == 3 ? lv.tz : 1, per = kz / split;
   t.kk0 = (bx % split) * per;
   t.nk = per;
   return t;
}

/* the split for a launch over n tiles of a level: the smallest power of
 * two dividing the tile depth that gives at least 1216 CTAs (8 per SM) */
static inline int split_for(const pgb_dlevel &lv, int n)
{
   const int kz = lv.dim == 3 ? lv.tz : 1;
   int sp = 1;
   while (sp < kz && (long)n * sp < 1216) sp *= 2;
   return sp;
}

/* FP32 <-> FP64 conversions in integer arithmetic. A conversion
 * instruction issues on the FP64 pipe, which runs at 1/64 of the FP32 rate
 * here; these take the integer pipes instead. f2d is exact except that FP32
 * subnormals (below 1.2e-38) become 0; d2f rounds toward zero (relative error
 * below 2^-23) and flushes results below the FP32 normal range to 0. Both
 * only touch values that steer the FP32 smoother or enter an FP64 sum as a
 * correction. */
__device__ __forceinline__ double f2d(float f)
{
   const unsigned int b = __float_as_uint(f);
   const unsigned int e = (b >> 23) & 0xffu;
   const unsigned long long sgn = (unsigned long long)(b >> 31) << 63;
   const unsigned long long ed = e == 0xffu ? 2047ull : (unsigned long long)(e + 896u);
   const unsigned long long v = sgn | (ed << 52) | ((unsigned long long)(b & 0x7fffffu) << 29);
   return __longlong_as_double((long long)(e ? v : sgn));
}

__device__ __forceinline__ float d2f(double d)
{
   const unsigned long long b = (unsigned long long)__double_as_longlong(d);
   const unsigned int hi = (unsigned int)(b >> 32), lo = (unsigned int)b;
   const int e = (int)((hi >> 20) & 0x7ffu) - 896;       /* FP32 biased exponent */
   const unsigned int sgn = hi & 0x80000000u;
   const unsigned int m = ((hi & 0xfffffu) << 3) | (lo >> 29);
   unsigned int r = sgn | ((unsigned int)e << 23) | m;
   r = e <= 0 ? sgn : r;
   r = e >= 255 ? (sgn | 0x7f800000u | (((hi >> 20) & 0x7ffu) == 0x7ffu && (m | (hi & 0xfffffu) | lo) ? 0x400000u : 0u)) : r;
   return __uint_as_float(r);
}

/* lap u in FP64 (num.f:113-115 up to rounding). Per dimension
 * RN(u+ - 2u) + u- rounds once at the scale of u (the last add is exact
 * near convergence, Sterbenz), which keeps the residual's rounding floor at
 * the reference's; summing the neighbours first would raise it. */
__device__ __forceinline__ double lapm(const pgb_dbox &b, const double *u, long p, long sy, long sz,
                                       int dim)
{
   const double c = u[p];
   const double dx = fma(-2.0, c, u[p + 1]) + u[p - 1];
   const double dy = fma(-2.0, c, u[p + sy]) + u[p - sy];
   if (b.flags & PGB_BOX_ISO) {
      if (dim == 3) return ((dx + dy) + (fma(-2.0, c, u[p + sz]) + u[p - sz])) * b.idx2[0];
      return (dx + dy) * b.idx2[0];
   }
   double t = fma(dy, b.idx2[1], dx * b.idx2[0]);
   if (dim == 3) t = fma(fma(-2.0, c, u[p + sz]) + u[p - sz], b.idx2[2], t);
   return t;
}

/* lapm with the centre and the two z neighbours supplied by the caller
 * (a thread walking its tile's planes keeps them in registers) */
__device__ __forceinline__ double lapw(const pgb_dbox &b, const double *u, long p, long sy, double c,
                                       double zm, double zp, int dim)
{
   const double dx = fma(-2.0, c, u[p + 1]) + u[p - 1];
   const double dy = fma(-2.0, c, u[p + sy]) + u[p - sy];
   if (b.flags & PGB_BOX_ISO) {
      if (dim == 3) return ((dx + dy) + (fma(-2.0, c, zp) + zm)) * b.idx2[0];
      return (dx + dy) * b.idx2[0];
   }
   double t = fma(dy, b.idx2[1], dx * b.idx2[0]);
   if (dim == 3) t = fma(fma(-2.0, c, zp) + zm, b.idx2[2], t);
   return t;
}

/* L[u] from lap u for the three operators (Poisson t - s, conformal factor
 * t + 2 pi s u^5, lapse t - s u; num.f:85-123 pattern) and, in c, the FP32
 * derivative of the non-Laplacian part (5 * 2 pi s u^4, -s, 0) */
template <bool PROG, bool VARS = false>
__device__ __forceinline__ double opjac(int pde, const pgb_dbox &b, long p, double t, double uc, double s,
                                        float &c)
{
   if (PROG && VARS) {   /* one variable of several, over its view of the boxes */
      if (!b.op->jfixed) c = d2f(__dsub_rn(pgb_prog_Jview(b, uc, s, p), b.j0));   /* else k_couplings' */
      return pgb_prog_Lview(b, t, uc, s, p);
   }
   if (PROG) {   /* an application's operator program (pgb_op.cuh) */
      c = d2f(__dsub_rn(pgb_prog_J(b, uc, s, p), b.j0));
      return pgb_prog_L(b, t, uc, s, p);
   }
   if (pde == 1) {
      double p2 = uc * uc, a = TWO_PI * s * (p2 * p2);
      c = 5.f * d2f(a);
      return fma(a, uc, t);
   }
   if (pde == 2) {
      c = -d2f(s);
      return fma(-s, uc, t);
   }
   c = 0.f;
   return t - s;
}

/* Several elliptic variables: the coupling coefficients dL/du_k of the
 * variable a box table's view holds, for the variables in slots
 * k = 1..nvread-1, at FP32 point q (the coupled colour pass k_relax32_vars
 * reads them). Out of line so that the one-variable instantiations keep
 * their registers. */
__device__ __noinline__ void store_coupling(const pgb_dop *o, double j0, double lapv, double u, const double *u1,
                                            const double *u2, const double *u3, pgb_srcv sv, float *out,
                                            long stride)
{
   double uv[PGB_NVAR_MAX];
   uv[0] = u;
   uv[1] = *u1;
   uv[2] = o->nvread > 2 ? *u2 : 0.0;
   uv[3] = o->nvread > 3 ? *u3 : 0.0;
   for (int k = 1; k < PGB_NVAR_MAX; k++)
      if (k < o->nvread) out[(k - 1) * stride] = d2f(pgb_prog_dvar(o->lcode, o->cst, lapv, j0, u, uv, sv, k));
}

__device__ __forceinline__ void coupling_at(const pgb_dbox &b, long p, long q, double lapv, double u, double s0,
                                            bool fill = false)
{
   const pgb_dop *o = b.op;
   if (o->nvread < 2 || (o->cfixed && !fill)) return;   /* fixed ones: k_couplings, once per prepare */
   const int nr = o->nvread;
   store_coupling(o, b.j0, lapv, u, b.f[PGB_FV(1, PGB_F_U)] + p, nr > 2 ? b.f[PGB_FV(2, PGB_F_U)] + p : 0,
                  nr > 3 ? b.f[PGB_FV(3, PGB_F_U)] + p : 0, pgb_load_src(o->nsrc, b, p, s0), b.w32c + q,
                  b.wz * b.n[2]);
}

/* The coupling coefficients (pgb_dop.cfixed) and the Jacobian term C
 * (pgb_dop.jfixed) of a level where they do not depend on the state: every
 * relaxed point of the view's variable */
__global__ void __launch_bounds__(NT) k_couplings(const pgb_dbox *boxes, pgb_dlevel lv)
{
   const pgb_tile tl = lv.tiles[blockIdx.x];
   const pgb_dbox b = boxes[tl.box];
   const int dim = lv.dim;
   const int i = tl.i0 + threadIdx.x, j = tl.j0 + threadIdx.y;
   const int kz = dim == 3 ? lv.tz : 1;
   if (i >= b.n[0] || j >= b.n[1]) return;
   const long sy = b.n[0], sz = (long)b.n[0] * b.n[1];
   for (int kk = 0; kk < kz; kk++) {
      const int k = tl.k0 + kk;
      if (k >= b.n[2]) break;
      const long p = i + sy * j + sz * k;
      if (!relaxed32(b, i, j, k, p, dim)) continue;
      const double *u = b.f[PGB_F_U];
      const long q = wq(b, i, j, k);
      if (b.op->cfixed) coupling_at(b, p, q, lapm(b, u, p, sy, sz, dim), u[p], b.f[PGB_F_SRC][p], true);
      if (b.op->jfixed) b.w32[W_C][q] = d2f(__dsub_rn(pgb_prog_Jview(b, u[p], b.f[PGB_F_SRC][p], p), b.j0));
   }
}

/* Down sweep, levels below the finest: app_L_op + compute_MG_rhs
 * (amrd/mg.c:271-314) fused with the FP64 defect of the pre-smoothing block:
 *     rhs = cmask_child ? -res*w0_r + L[u] : 0,   lop = u,
 *     D = rhs - L[u], C at relaxed points.
 * E is 0 on entry (every block ends by clearing it). With cover = 1 only
 * the level's cover tiles are visited: elsewhere rhs stays 0 and D is the
 * FP32 update k_defect32 made at the end of the previous post-smoothing. */
template <bool PROG, bool TAIL, bool VARS = false>
__device__ __forceinline__ void fas_defect_b(const vblk &vb, const pgb_dbox *boxes, const pgb_dlevel &lv, int pde,
                                             double w0_r, int cover, int split)
{
   const tile_part tp = tile_split(cover ? lv.ctiles : lv.tiles, lv, split, vb.x);
   const pgb_tile tl = tp.tl;
   const pgb_dbox b = boxes[tl.box];
   const int dim = lv.dim;
   const int i = tl.i0 + threadIdx.x, j = tl.j0 + threadIdx.y;
   if (i >= b.n[0] || j >= b.n[1]) return;
   RP(const double) u = b.f[PGB_F_U];
   RP(const double) src = b.f[PGB_F_SRC];
   RP(const double) res = b.f[PGB_F_RES];
   RP(double) rhs = b.f[PGB_F_RHS];
   RP(double) lop = b.f[PGB_F_LOP];
   RP(float) wd = b.w32[W_D];
   RP(float) wc = b.w32[W_C];
   const long sy = b.n[0], sz = (long)b.n[0] * b.n[1];
   const int ks = tl.k0 + tp.kk0;
   if (ks >= b.n[2]) return;
   long p = i + sy * j + sz * ks, q = wq(b, i, j, ks);
   double zm = (dim == 3 && ks > 0) ? u[p - sz] : 0.0, uc = u[p];
#pragma unroll
   for (int kk = 0; kk < PGB_TZ; kk++, p += sz, q += b.wz) {
      const int k = ks + kk;
      if (kk >= tp.nk || k >= b.n[2]) continue;
      const double zp = (dim == 3 && k + 1 < b.n[2]) ? u[p + sz] : 0.0;
      const int cm = b.cmask_child[p];
      const bool in = interior32(b, i, j, k, dim);
      const bool rl = in && ((b.flags & PGB_BOX_BDY_INTERIOR) || b.cmask_bdy[p]);
      double r = 0.0;
      if (in && (cm || rl)) {
         float c;
         const double lp = lapw(b, u, p, sy, uc, zm, zp, dim);
         const double l = opjac<PROG, VARS>(pde, b, p, lp, uc, src[p], c);
         if (cm) r = fma(-res[p], w0_r, l);
         if (rl) {
            wd[q] = d2f(r - l);
            if (!VARS || !b.op->jfixed) wc[q] = c;
            if (VARS) coupling_at(b, p, q, lp, uc, src[p]);
         }
      } else if (cm)
         r = -res[p] * w0_r;
      rhs[p] = r;
      lop[p] = uc;
      zm = uc;
      uc = zp;
   }
}

template <bool PROG, bool VARS = false>
__global__ void __launch_bounds__(NT) k_fas_defect(const pgb_dbox *boxes, pgb_dlevel lv, int pde,
                                                   double w0_r, int cover, int split)
{
   fas_defect_b<PROG, false, VARS>(hw_blk(), boxes, lv, pde, w0_r, cover, split);
}

/* The Gauss-Seidel update of one point of lap E + C E = D, FP32, written
 * with explicit roundings so that every kernel that relaxes (colour passes
 * from global memory, fused sweeps in shared memory) computes the same
 * bits: t = sum over dimensions of (e+ - 2 e + e-) * idx2 (the first a
 * product, the others fused), r = (c e + t) - d, e - r / (j0 + c). */
__device__ __forceinline__ float gs32(float ec, float xm, float xp, float ym, float yp, float zm, float zp,
                                      float c, float d, float ix, float iy, float iz, float j0, bool d3)
{
   const float m2 = -2.f * ec;   /* exact */
   float t = __fmul_rn(__fadd_rn(__fadd_rn(xp, m2), xm), ix);
   t = __fmaf_rn(__fadd_rn(__fadd_rn(yp, m2), ym), iy, t);
   if (d3) t = __fmaf_rn(__fadd_rn(__fadd_rn(zp, m2), zm), iz, t);
   const float r = __fsub_rn(__fmaf_rn(c, ec, t), d);
   return __fsub_rn(ec, __fdividef(r, __fadd_rn(j0, c)));
}

/* one colour pass of Gauss-Seidel on lap E + C E = D, FP32, straight from
 * global memory (the level's E, D, C stay in L2 between passes); relax
 * tiles are 64 points wide, a thread updates one point of the active colour
 * per row (parity as num.f:220) */
template <bool TAIL>
__device__ __forceinline__ void relax32_b(const vblk &vb, const pgb_dbox *boxes, const pgb_dlevel &lv, int pass)
{
   const pgb_tile tl = lv.rtiles[vb.x];
   const pgb_dbox b = boxes[tl.box];
   const int dim = lv.dim;
   RP(float) e = b.w32[W_E];
   RP(const float) dd = b.w32[W_D];
   RP(const float) cc = b.w32[W_C];
   const long sy = b.n[0], sz = (long)b.n[0] * b.n[1], wy = b.wy, wz = b.wz;
   const float ix = b.fidx2[0], iy = b.fidx2[1], iz = b.fidx2[2];
   const float j0 = b.fj0;
   const int j = tl.j0 + threadIdx.y;
   const int kz = dim == 3 ? lv.rtz : 1;
#pragma unroll
   for (int kk = 0; kk < PGB_TZ; kk++) {
      if (kk >= kz) continue;
      const int k = tl.k0 + kk;
      const int par = dim == 3 ? ((j + k + 1 + pass) & 1) : ((j + pass) & 1);
      const int i = tl.i0 + 2 * threadIdx.x + par;
      if (!interior32(b, i, j, k, dim)) continue;
      const long p = i + sy * j + sz * k, q = i + wy * j + wz * k;
      if (!(b.flags & PGB_BOX_BDY_INTERIOR) && !b.cmask_bdy[p]) continue;
      const bool d3 = dim == 3;
      e[q] = gs32(e[q], e[q - 1], e[q + 1], e[q - wy], e[q + wy], d3 ? e[q - wz] : 0.f, d3 ? e[q + wz] : 0.f,
                  cc[q], dd[q], ix, iy, iz, j0, d3);
   }
}

__global__ void __launch_bounds__(NT) k_relax32(const pgb_dbox *boxes, pgb_dlevel lv, int pass)
{
   relax32_b<false>(hw_blk(), boxes, lv, pass);
}

/* One colour pass of the coupled FP32 smoother of several elliptic
 * variables: at each point of the colour, variable 0, 1, ... in turn, each
 * from the others' current corrections at the point (the point-wise order
 * of the FP64 form's relax over the variables), on
 *     lap E_v + C_v E_v + sum_k C_vk E_k = D_v
 * with C_vk the coupling coefficients of the FP64 passes (w32c, slot k of
 * variable v's view holding variable k, or 0 where k = v). In place on
 * each variable's E; vt.t[v] is variable v's view of the boxes. */
__global__ void __launch_bounds__(NT) k_relax32_vars(pgb_vtabs vt, pgb_dlevel lv, int pass)
{
   const pgb_tile tl = lv.rtiles[blockIdx.x];
   const pgb_dbox b = vt.t[0][tl.box];
   const int dim = lv.dim, nv = lv.nvar;
   const long sy = b.n[0], sz = (long)b.n[0] * b.n[1], wy = b.wy, wz = b.wz, cs = b.wz * b.n[2];
   const float ix = b.fidx2[0], iy = b.fidx2[1], iz = b.fidx2[2];
   const float j0 = b.fj0;
   const int j = tl.j0 + threadIdx.y;
   const int kz = dim == 3 ? lv.rtz : 1;
   /* every variable's arrays, in registers (the loops over the variables
    * unroll, so the indices are constants) */
   float *ev[PGB_NVAR_MAX];
   const float *cv[PGB_NVAR_MAX], *dv[PGB_NVAR_MAX], *kv[PGB_NVAR_MAX];
#pragma unroll
   for (int v = 0; v < PGB_NVAR_MAX; v++) {
      const pgb_dbox *bv = v < nv ? &vt.t[v][tl.box] : 0;
      ev[v] = bv ? bv->w32[W_E] : 0;
      cv[v] = bv ? bv->w32[W_C] : 0;
      dv[v] = bv ? bv->w32[W_D] : 0;
      kv[v] = bv ? bv->w32c : 0;
   }
   for (int kk = 0; kk < PGB_TZ; kk++) {
      if (kk >= kz) break;
      const int k = tl.k0 + kk;
      const int par = dim == 3 ? ((j + k + 1 + pass) & 1) : ((j + pass) & 1);
      const int i = tl.i0 + 2 * threadIdx.x + par;
      if (!interior32(b, i, j, k, dim)) continue;
      const long p = i + sy * j + sz * k, q = i + wy * j + wz * k;
      if (!(b.flags & PGB_BOX_BDY_INTERIOR) && !b.cmask_bdy[p]) continue;
      const bool d3 = dim == 3;
#pragma unroll
      for (int v = 0; v < PGB_NVAR_MAX; v++) {
         if (v >= nv) break;
         float off = 0.f;
#pragma unroll
         for (int k2 = 1; k2 < PGB_NVAR_MAX; k2++)
            if (k2 < nv) off = __fmaf_rn(kv[v][(k2 - 1) * cs + q], ev[k2 == v ? 0 : k2][q], off);
         float *e = ev[v];
         e[q] = gs32(e[q], e[q - 1], e[q + 1], e[q - wy], e[q + wy], d3 ? e[q - wz] : 0.f, d3 ? e[q + wz] : 0.f,
                     cv[v][q], __fsub_rn(dv[v][q], off), ix, iy, iz, j0, d3);
      }
   }
}

/* The same sweeps staged in shared memory: NS red-black sweeps in one launch.
 * The CTA stages the correction of its 32 x 8 x tz tile plus a halo of
 * 2*NS points from slot `src` in shared memory; colour pass q (0 ..
 * 2*NS-1) updates the active colour on the tile grown by 2*NS-1-q points,
 * so that every value the next pass reads is already final, and only the
 * tile is written, to slot `dst`. A point's new value depends only on old
 * values of the other colour and D, C, so neighbouring CTAs compute
 * identical values on their overlaps; since no CTA writes the slot the
 * others stage from, the halo is the old correction whatever the CTAs'
 * order, and the result is that of the in-place colour passes bit for bit.
 * Colour of pass q: the points with i+j(+k+1)+q even (num.f:220 parity,
 * 0-based indices). NS > 1 is only used on levels with no sync between
 * sweeps. */
template <int NS>
__global__ void __launch_bounds__(NT) k_sweep32(const pgb_dbox *boxes, pgb_dlevel lv, int src, int dst)
{
   constexpr int H = 2 * NS;
   constexpr int SX = PGB_TX + 2 * H, SY = PGB_TY + 2 * H, SZ = PGB_TZ + 2 * H;
   __shared__ float se[SZ * SY * SX];
   const pgb_tile tl = lv.tiles[blockIdx.x];
   const pgb_dbox b = boxes[tl.box];
   const int dim = lv.dim;
   const int tz = dim == 3 ? lv.tz : 1, hz = dim == 3 ? H : 0, nzl = tz + 2 * hz;
   const long sy = b.n[0], sz = (long)b.n[0] * b.n[1];
   const float *e = eslot(b, src);
   float *eo = eslot(b, dst);
   const float *dd = b.w32[W_D], *cc = b.w32[W_C];
   const float ix = b.fidx2[0], iy = b.fidx2[1], iz = b.fidx2[2];
   const float j0 = b.fj0;
   const bool allbdy = b.flags & PGB_BOX_BDY_INTERIOR;
   const int t = threadIdx.x + threadIdx.y * PGB_TX;
   const int gi0 = tl.i0 - H, gj0 = tl.j0 - H, gk0 = tl.k0 - hz;
   for (int q = t; q < SX * SY * nzl; q += NT) {
      const int x = q % SX, y = (q / SX) % SY, z = q / (SX * SY);
      const int gi = gi0 + x, gj = gj0 + y, gk = gk0 + z;
      float v = 0.f;
      if (gi >= 0 && gi < b.n[0] && gj >= 0 && gj < b.n[1] && gk >= 0 && gk < b.n[2])
         v = e[wq(b, gi, gj, gk)];
      se[x + SX * (y + SY * z)] = v;
   }
   __syncthreads();
#pragma unroll
   for (int pass = 0; pass < 2 * NS; pass++) {
      const int g = H - 1 - pass;                    /* growth of this pass's region */
      const int gz = dim == 3 ? g : 0;
      const int rx = PGB_TX + 2 * g, ry = PGB_TY + 2 * g, rz = tz + 2 * gz;
      const int hx = (rx + 1) / 2;                   /* slots per row: every other point */
      for (int q = t; q < hx * ry * rz; q += NT) {
         const int xs = q % hx, yy = (q / hx) % ry, zz = q / (hx * ry);
         const int y = H - g + yy, z = hz - gz + zz;
         const int gj = gj0 + y, gk = gk0 + z;
         const int xstart = H - g;
         /* first x of the row with the active colour */
         const int par = ((gi0 + xstart + gj + (dim == 3 ? gk + 1 : 0) + pass) & 1);
         const int x = xstart + par + 2 * xs;
         if (x >= xstart + rx) continue;
         const int gi = gi0 + x;
         if (!interior32(b, gi, gj, gk, dim)) continue;
         const long p = gi + sy * gj + sz * gk;
         if (!allbdy && !b.cmask_bdy[p]) continue;
         const int sp = x + SX * (y + SY * z);
         const bool d3 = dim == 3;
         const long qw = wq(b, gi, gj, gk);
         se[sp] = gs32(se[sp], se[sp - 1], se[sp + 1], se[sp - SX], se[sp + SX], d3 ? se[sp - SX * SY] : 0.f,
                       d3 ? se[sp + SX * SY] : 0.f, cc[qw], dd[qw], ix, iy, iz, j0, d3);
      }
      __syncthreads();
   }
   for (int q = t; q < PGB_TX * PGB_TY * tz; q += NT) {
      const int x = q % PGB_TX, y = (q / PGB_TX) % PGB_TY, z = q / (PGB_TX * PGB_TY);
      const int gi = tl.i0 + x, gj = tl.j0 + y, gk = tl.k0 + z;
      if (gi < b.n[0] && gj < b.n[1] && gk < b.n[2])
         eo[wq(b, gi, gj, gk)] = se[(x + H) + SX * ((y + H) + SY * (z + hz))];
   }
}

/* One red-black sweep in one pass over memory (3-D levels): the CTA owns a
 * 32 x 8 column of ztz planes (a ztile) and marches through it, two planes
 * per step. Planes of the old correction (slot src), D and C, each with a
 * halo of two points, stream into 8-plane rings in shared memory by
 * cp.async, one step ahead of use. Step k (k, k+1 landed): the first colour
 * of planes k-1 and k on the column grown by one point (from old
 * second-colour values), then the second colour of planes k-2 and k-1 on
 * the column (from the new first-colour values of the planes around them),
 * then planes k-2 and k-1 are written to slot dst. The first colour of the
 * planes just outside the chunk is recomputed for the purpose; as in
 * k_sweep32 no CTA writes the slot the others read, so every value equals
 * that of the in-place colour passes bit for bit. Traffic: each array once
 * per sweep (16 B per point) plus halo re-reads, against two passes over
 * every array for the colour-pass kernels. */
#define ZX (PGB_TX + 4)
#define ZY (PGB_TY + 4)
#define ZR 8            /* ring depth (planes) */

__device__ __forceinline__ void cp_async4(uint32_t dst, const float *src, bool valid)
{
   asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(dst), "l"(src), "r"(valid ? 4 : 0) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

__global__ void __launch_bounds__(NT) k_sweep32z(const pgb_dbox *boxes, pgb_dlevel lv, int src, int dst)
{
   constexpr int PL = ZX * ZY;   /* floats per staged plane */
   __shared__ float se[ZR * PL], sd[ZR * PL], sc[ZR * PL];
   const pgb_tile tl = lv.ztiles[blockIdx.x];
   const pgb_dbox *bp = boxes + tl.box;
   const int n0 = bp->n[0], n1 = bp->n[1], n2 = bp->n[2];
   const long sz = (long)n0 * n1;
   const float *__restrict__ e = bp->w32[src];
   float *__restrict__ eo = bp->w32[dst];
   const float *__restrict__ dd = bp->w32[W_D];
   const float *__restrict__ cc = bp->w32[W_C];
   const uint8_t *__restrict__ cmb = (bp->flags & PGB_BOX_BDY_INTERIOR) ? nullptr : bp->cmask_bdy;
   const float ix = bp->fidx2[0], iy = bp->fidx2[1], iz = bp->fidx2[2];
   const float j0 = bp->fj0;
   const int t = threadIdx.x + threadIdx.y * PGB_TX;
   const int gi0 = tl.i0 - 2, gj0 = tl.j0 - 2;
   const int k0 = tl.k0, k1 = min(tl.k0 + lv.ztz, n2);   /* planes [k0, k1) written */

   /* what a thread does is the same on every plane: its staged points (two
    * at most), its point of each colour pass for both parities, and its
    * store, as offsets within a plane */
   const uint32_t ue = (uint32_t)__cvta_generic_to_shared(se), ud = (uint32_t)__cvta_generic_to_shared(sd),
                  uc = (uint32_t)__cvta_generic_to_shared(sc);
   int lso[2], lgo[2];
   bool lin[2], lany[2];
#pragma unroll
   for (int u = 0; u < 2; u++) {
      const int q = t + u * NT, x = q % ZX, y = q / ZX, gi = gi0 + x, gj = gj0 + y;
      lany[u] = q < PL;
      lin[u] = lany[u] && gi >= 0 && gi < n0 && gj >= 0 && gj < n1;
      lso[u] = 4 * q;
      lgo[u] = lin[u] ? gi + bp->wy * gj : 0;   /* FP32 arrays: padded pitch */
   }
   int rso[2][2], rgo[2][2], rpar[2];   /* [pass][parity] */
   bool rok[2][2];
#pragma unroll
   for (int pass = 0; pass < 2; pass++) {
      const int grow = 1 - pass, w = PGB_TX + 2 * grow, h = PGB_TY + 2 * grow, slots = (w + 1) / 2;
      const int y = 2 - grow + t / slots, gj = gj0 + y, xs = 2 - grow;
      rpar[pass] = (gi0 + xs + gj + 1 + pass) & 1;   /* parity at plane 0; flips with the plane */
#pragma unroll
      for (int par = 0; par < 2; par++) {
         const int x = xs + par + 2 * (t % slots), gi = gi0 + x;
         rok[pass][par] = t < slots * h && x < xs + w && gi >= 1 && gi <= n0 - 2 && gj >= 1 && gj <= n1 - 2;
         rso[pass][par] = y * ZX + x;
         rgo[pass][par] = rok[pass][par] ? gi + n0 * gj : 0;
      }
   }
   const int sxs = 2 + t % PGB_TX, sys_ = 2 + t / PGB_TX;
   const bool sok = gi0 + sxs < n0 && gj0 + sys_ < n1;
   const int sso = sys_ * ZX + sxs;
   const long sgo = (long)(gi0 + sxs) + (long)bp->wy * (gj0 + sys_);

   auto fetch = [&](int k) {   /* plane k's copies (none outside the box or past what the chunk reads) */
      if (k < 0 || k >= n2 || k > k1 + 1) return;
      const long koff = bp->wz * k;
      const uint32_t r = 4u * (uint32_t)((k & (ZR - 1)) * PL);
#pragma unroll
      for (int u = 0; u < 2; u++)
         if (lany[u]) {
            const long g = lin[u] ? koff + lgo[u] : 0;
            cp_async4(ue + r + lso[u], e + g, lin[u]);
            cp_async4(ud + r + lso[u], dd + g, lin[u]);
            cp_async4(uc + r + lso[u], cc + g, lin[u]);
         }
   };
   /* colour `pass` of plane kp */
   auto relax = [&](int pass, int kp) {
      const bool active = pass == 0 ? (kp >= k0 - 1 && kp <= k1) : (kp >= k0 && kp < k1);
      const bool odd = (rpar[pass] + kp) & 1;   /* registers, not an indexed array */
      const bool ok = odd ? rok[pass][1] : rok[pass][0];
      const int o = odd ? rso[pass][1] : rso[pass][0], go = odd ? rgo[pass][1] : rgo[pass][0];
      if (active && kp >= 1 && kp <= n2 - 2 && ok && (!cmb || cmb[go + sz * kp])) {
         const int r = (kp & (ZR - 1)) * PL;
         const float *m = se + ((kp - 1) & (ZR - 1)) * PL, *pl = se + ((kp + 1) & (ZR - 1)) * PL;
         float *c = se + r;
         c[o] = gs32(c[o], c[o - 1], c[o + 1], c[o - ZX], c[o + ZX], m[o], pl[o], sc[r + o], sd[r + o], ix, iy, iz,
                     j0, true);
      }
   };

   fetch(k0 - 2);
   fetch(k0 - 1);
   cp_async_commit();
   for (int k = k0 - 2; k <= k1 + 1; k += 2) {
      cp_async_wait_all();   /* planes k, k+1 */
      __syncthreads();
      fetch(k + 2);
      fetch(k + 3);
      cp_async_commit();
      relax(0, k - 1);
      relax(0, k);
      __syncthreads();
      relax(1, k - 2);
      relax(1, k - 1);
      __syncthreads();
#pragma unroll
      for (int kw = k - 2; kw < k; kw++)   /* planes finished at this step */
         if (kw >= k0 && kw < k1 && sok) eo[sgo + bp->wz * kw] = se[(kw & (ZR - 1)) * PL + sso];
   }
   cp_async_wait_all();
}
#undef ZX
#undef ZY
#undef ZR

/* ------------------------------------------- one-pass sweep, TMA-staged -- */
/* One red-black sweep in one pass over memory on 3-D levels, the planes
 * staged by the Tensor Memory Accelerator. A CTA owns an output column of
 * TXO x TYO points (x start a multiple of 4, so that every TMA load starts
 * on 16 bytes: the FP32 rows are padded to 16-byte pitches) and marches
 * through MTZ planes of it (MTZ even). Each plane of the old correction
 * (slot src, TXO+8 x TYO+4 points around the column), of D and of C
 * (TXO+8 x TYO+2) arrives by one cp.async.bulk.tensor 3-D tile load per
 * array into a ring of R = 8 plane slots, completion counted on the slot's
 * mbarrier; loads run R-2 planes ahead of use and fill out-of-box
 * coordinates with zeros.
 *
 * Each thread owns a point pair (x, x+1) of one row y of the column grown by
 * one point, with x + y even, so that at plane k the first colour (num.f:220
 * parity, 0-based: x + y + k odd) is the pair's first member for odd k and
 * its second for even k, for every thread alike. At plane step k a thread
 * updates its member c of the first colour at (c, k), from the old
 * second-colour values around it, then the second colour at (c, k-1),
 * whose z neighbours are the new first-colour values at (c, k-2) and (c, k)
 * it computed two steps ago and just now, whose x neighbour inside the pair
 * is the other member's new value at k-1 (one step ago), and whose old value
 * is the z neighbour the first-colour update read. The old values at
 * (other member, k) and (c, k-1) are the ones the previous step loaded as
 * its z and x neighbours. Only first-colour results go to shared memory
 * (the neighbours read them one step later); plane k-1 is final after the
 * second-colour update and is stored from registers. Within a step no
 * thread reads what another writes, so one barrier per step suffices; it
 * also frees plane k-1's slot for the load of plane k-1+R. The loop is
 * unrolled over the ring, so that slots and colours are constants and every
 * shared-memory access is one register plus an immediate; the two
 * half-warps of a warp hold neighbouring rows (whose pairs start one point
 * apart), which keeps the stride-2 accesses free of bank conflicts.
 *
 * No CTA writes the slot the others read and every update is gs32 on the
 * same operands, so the result equals the in-place colour passes bit for
 * bit. Every mbarrier wait is bounded (globaltimer, ~1 s); on timeout the
 * CTA sets *err, lets the loads it issued land and returns. Boxes must have
 * their whole interior relaxed (PGB_BOX_BDY_INTERIOR). */
#define MT_R 8           /* ring slots (planes); the step loop is unrolled over them */
#define MT_TYO 14        /* output rows per column */
#define MT_NMAPS 16      /* tensor maps per box: 4 per column width (60, 28 one sweep; 24, 56 two) */

__device__ __forceinline__ uint32_t mt_saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t mt_ns()
{
   uint64_t t;
   asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
   return t;
}

__device__ __forceinline__ bool mt_try(uint64_t *bar, uint32_t phase)
{
   uint32_t ok;
   asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                " selp.u32 %0, 1, 0, p;\n}\n"
                : "=r"(ok)
                : "r"(mt_saddr(bar)), "r"(phase)
                : "memory");
   return ok != 0;
}

/* bounded wait for the phase of parity `phase`; the clock is read only when
 * the first try fails */
__device__ __forceinline__ bool mt_wait(uint64_t *bar, uint32_t phase)
{
   if (mt_try(bar, phase)) return true;
   const uint64_t t0 = mt_ns();
   while (!mt_try(bar, phase))
      if (mt_ns() - t0 > 1000000000ull) return false;
   return true;
}

/* 3-D tile of a tensor map into shared memory, completion on bar */
__device__ __forceinline__ void mt_load(float *dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar)
{
   asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(mt_saddr(dst)),
                "l"((unsigned long long)map), "r"(x), "r"(y), "r"(z), "r"(mt_saddr(bar))
                : "memory");
}

template <int TXO>
struct mt_shape {
   static constexpr int PX = (TXO + 4) / 2, PY = MT_TYO + 2, NTH = PX * PY, HX = PX / 16;
   static constexpr int EW = TXO + 8, EH = MT_TYO + 4, DH = MT_TYO + 2;
   static constexpr int ESZ = (EW * EH + 31) / 32 * 32, DSZ = (EW * DH + 31) / 32 * 32;
   static constexpr int SLOT = ESZ + 2 * DSZ;                 /* floats per ring slot (128-byte multiple) */
   static constexpr unsigned EBYTES = 4u * EW * EH, DBYTES = 4u * EW * DH;
   static constexpr size_t SMEM = 4ul * MT_R * SLOT + 8ul * MT_R;
   static constexpr int MINB = TXO >= 60 ? 2 : 3;             /* CTAs per SM the shared memory allows */
   static_assert(PX % 16 == 0 && PY % 2 == 0, "half-warps hold 16 pairs of one row");
};

template <int TXO>
__global__ void __launch_bounds__(mt_shape<TXO>::NTH, mt_shape<TXO>::MINB)
   k_sweep32t(const pgb_dbox *boxes, pgb_dlevel lv, const CUtensorMap *maps, int src, int dst, int *err)
{
   typedef mt_shape<TXO> S;
   constexpr int EW = S::EW, SL = S::SLOT, DO = S::ESZ - EW, CO = S::ESZ + S::DSZ - EW;   /* D, C of a point: +DO, +CO */
   extern __shared__ __align__(128) float sm[];
   uint64_t *bar = (uint64_t *)(sm + MT_R * SL);
   const pgb_tile tl = lv.mtiles[blockIdx.x];
   const pgb_dbox *bp = boxes + tl.box;
   const int n0 = bp->n[0], n1 = bp->n[1], n2 = bp->n[2];
   const float ix = bp->fidx2[0], iy = bp->fidx2[1], iz = bp->fidx2[2], j0 = bp->fj0;
   const CUtensorMap *me = maps + MT_NMAPS * tl.box + (src == W_E2 ? 1 : 0), *md = maps + MT_NMAPS * tl.box + 2,
                     *mc = maps + MT_NMAPS * tl.box + 3;
   const int i0 = tl.i0, jb = tl.j0, kb = tl.k0, ke = min(tl.k0 + lv.mtz, n2);   /* planes [kb, ke) written */
   if (kb & 1) {   /* the unrolled colours assume an even first plane */
      if (threadIdx.x == 0) *err = 2;
      return;
   }
   const int t = threadIdx.x, w = t >> 5;
   const int tx = (w % S::HX) * 16 + (t & 15), ty = 2 * (w / S::HX) + ((t >> 4) & 1);
   const int gy = jb - 1 + ty, xs = i0 - 2 + 2 * tx + (gy & 1);   /* the pair: (xs, xs+1) of row gy, xs + gy even */
   float *const s0 = sm + (1 + ty) * EW + 2 + 2 * tx + (gy & 1);  /* the first member in slot 0's E plane */
   const bool yin = gy >= 1 && gy <= n1 - 2;
   const bool xin0 = yin && xs >= 1 && xs <= n0 - 2, xin1 = yin && xs >= 0 && xs <= n0 - 3;
   /* first colour on x in [i0-1, i0+TXO]; second colour and the store on the output column */
   const bool rr0 = xs >= i0 - 1 && xs <= i0 + TXO, rr1 = xs + 1 >= i0 - 1 && xs + 1 <= i0 + TXO;
   const bool orow = ty >= 1 && ty <= S::PY - 2 && gy < n1;
   const bool out0 = orow && xs >= i0 && xs <= i0 + TXO - 1 && xs < n0;
   const bool out1 = orow && xs + 1 >= i0 && xs + 1 <= i0 + TXO - 1 && xs + 1 < n0;
   float *gp = bp->w32[dst] + (out0 || out1 ? xs + bp->wy * gy : 0);
   const long wz = bp->wz;
   if (t == 0) {
      for (int r = 0; r < MT_R; r++)
         asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mt_saddr(bar + r)), "r"(1) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
   }
   __syncthreads();
   /* plane m lives in slot (m - m0) % R; its phase parity flips with each reuse */
   const int m0 = kb - 2, mlast = min(ke + 1, n2 - 1);
   int last_issued = m0 - 1;   /* thread 0: the newest plane whose slot a load or arrival was issued for */
   auto issue = [&](int m) {   /* thread 0 */
      uint64_t *b = bar + ((m - m0) & (MT_R - 1));
      last_issued = m;
      if (m < 0 || m > mlast) {   /* nothing to load: complete the slot's phase anyway */
         asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mt_saddr(b)) : "memory");
         return;
      }
      float *sl = sm + ((m - m0) & (MT_R - 1)) * SL;
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mt_saddr(b)),
                   "r"(S::EBYTES + 2 * S::DBYTES) : "memory");
      mt_load(sl, me, i0 - 4, jb - 2, m, b);
      mt_load(sl + S::ESZ, md, i0 - 4, jb - 1, m, b);
      mt_load(sl + S::ESZ + S::DSZ, mc, i0 - 4, jb - 1, m, b);
   };
   if (t == 0)
      for (int m = m0; m < m0 + MT_R; m++) issue(m);
   /* planes kb-2 and kb-1 (slots 0 and 1) before the first step */
   bool ok = true;
   int waited = m0 - 1;   /* planes up to here have landed (each thread observes it itself) */
   for (int q = m0; q <= min(kb - 1, mlast); q++) {
      if (q >= 0 && !mt_wait(bar + (q - m0), 0)) ok = false;
      waited = q;
   }
   /* old values carried between steps: (other member, k) and (c, k-1) */
   float zprev = s0[SL + 1], aprev = s0[0];
   float rp1 = 0.f, rp2 = 0.f;   /* new first-colour values: (other member, k-1), (c, k-2) */
   gp += wz * (long)(kb - 3);   /* advanced to plane k-1 at each step */

   /* step s: plane k = kb - 1 + s, slot (s + 1) % R; colour member mem = s % 2 */
   for (int sb = 0;; sb += MT_R) {
      const uint32_t ph = (sb / MT_R) & 1;
#pragma unroll
      for (int u = 0; u < MT_R; u++) {
         const int s = sb + u, k = kb - 1 + s;
         if (k > ke) return;
         const int mem = u & 1;
         const int jk = ((u + 1) & (MT_R - 1)) * SL, jm = (u & (MT_R - 1)) * SL, jp = ((u + 2) & (MT_R - 1)) * SL;
         if (k + 1 <= mlast) {   /* plane k+1 in slot (s + 2) % R */
            if (!mt_wait(bar + ((u + 2) & (MT_R - 1)), ph ^ (u + 2 >= MT_R ? 1u : 0u))) ok = false;
            waited = k + 1;
         }
         float *pc = s0 + mem;   /* the member c of the first colour at plane k */
         /* first colour at (c, k) */
         const float ec = pc[jk], ea = zprev, ezm = aprev;
         const float eb = mem ? pc[jk + 1] : pc[jk - 1];
         const float zp = pc[jp];
         float rk = gs32(ec, mem ? ea : eb, mem ? eb : ea, pc[jk - EW], pc[jk + EW], ezm, zp, pc[jk + CO],
                         pc[jk + DO], ix, iy, iz, j0, true);
         if (!((mem ? xin1 : xin0) && k >= 1 && k <= n2 - 2)) rk = ec;
         if (mem ? rr1 : rr0) pc[jk] = rk;
         /* second colour at (c, k-1); then plane k-1 of the pair is final */
         gp += wz;
         if (s >= 2) {
            const float fb = mem ? pc[jm + 1] : pc[jm - 1];
            float bk = gs32(ezm, mem ? rp1 : fb, mem ? fb : rp1, pc[jm - EW], pc[jm + EW], rp2, rk, pc[jm + CO],
                            pc[jm + DO], ix, iy, iz, j0, true);
            if (!((mem ? xin1 : xin0) && k >= 2 && k <= n2 - 1)) bk = ezm;
            if (out0) gp[0] = mem ? rp1 : bk;
            if (out1) gp[1] = mem ? bk : rp1;
         }
         zprev = zp;
         aprev = ea;
         rp2 = rp1;
         rp1 = rk;
         if (!ok) *err = 1;
         if (__syncthreads_or(!ok)) {   /* a load never landed: let the issued ones land, return */
            if (t == 0)
               for (int q = max(waited + 1, 0); q <= min(mlast, last_issued); q++)
                  mt_wait(bar + ((q - m0) & (MT_R - 1)), ((q - m0) / MT_R) & 1);
            return;
         }
         /* plane k-1's slot is free: every thread is past step k */
         if (t == 0) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(k - 1 + MT_R);
         }
      }
   }
}

/* ----------------------------------- two sweeps per launch, TMA-staged -- */
/* Two red-black sweeps of k_sweep32t's kind in one pass over memory: the
 * second sweep trails the first by two planes inside the same CTA. A CTA
 * owns an output column of TXO x TYO points; the first sweep runs on the
 * column grown by 3 points (first colour) and 2 (second colour), the second
 * on the column grown by 1 (first colour) and the column itself (second
 * colour), so every value the second sweep reads is the first sweep's final
 * value, computed identically by the CTAs that share it. E is staged grown
 * by 4 points (TXO+8 x TYO+8), D and C by 3; plane slots live until the
 * second sweep's last read of them (planes k-3 .. k+1 at step k), so loads
 * run 4 planes ahead in the ring of 8.
 *
 * Each thread owns a point pair (x, x+1) of one row with x + y even, as in
 * k_sweep32t, and at step k works on the member c of the first colour at
 * plane k, which is also the first colour at k-2: first sweep, first
 * colour at (c, k) and second colour at (c, k-1) (written back to its slot,
 * where the second sweep reads it); second sweep, first colour at (c, k-2)
 * from the first sweep's final values (its z neighbours (c, k-3) and
 * (c, k-1) and its in-pair x neighbour are first-sweep second-colour values
 * this thread computed in the last three steps, registers), then second
 * colour at (c, k-3) (z neighbours and in-pair x neighbour: second-sweep
 * first-colour values of the last three steps), and plane k-3 of the pair
 * is final and stored from registers. Within a step no thread reads what
 * another writes, so one barrier per step suffices. Every update is gs32,
 * so the result equals two in-place sweeps of colour passes bit for bit.
 * Waits are bounded as in k_sweep32t. */
template <int TXO>
struct mt2_shape {
   static constexpr int PX = (TXO + 8) / 2, PY = MT_TYO + 6, NTH = PX * PY, HX = PX / 16;
   static constexpr int EW = TXO + 8, EH = MT_TYO + 8, DH = MT_TYO + 6;
   static constexpr int ESZ = (EW * EH + 31) / 32 * 32, DSZ = (EW * DH + 31) / 32 * 32;
   static constexpr int SLOT = ESZ + 2 * DSZ;
   static constexpr unsigned EBYTES = 4u * EW * EH, DBYTES = 4u * EW * DH;
   static constexpr size_t SMEM = 4ul * MT_R * SLOT + 8ul * MT_R;
   static constexpr int MINB = TXO >= 56 ? 1 : 3;
   static_assert(PX % 16 == 0 && PY % 2 == 0, "half-warps hold 16 pairs of one row");
};

template <int TXO>
__global__ void __launch_bounds__(mt2_shape<TXO>::NTH, mt2_shape<TXO>::MINB)
   k_sweep32t2(const pgb_dbox *boxes, pgb_dlevel lv, const CUtensorMap *maps, int src, int dst, int *err)
{
   typedef mt2_shape<TXO> S;
   constexpr int EW = S::EW, SL = S::SLOT, DO = S::ESZ - EW, CO = S::ESZ + S::DSZ - EW;
   extern __shared__ __align__(128) float sm[];
   uint64_t *bar = (uint64_t *)(sm + MT_R * SL);
   const pgb_tile tl = lv.mtiles[blockIdx.x];
   const pgb_dbox *bp = boxes + tl.box;
   const int n0 = bp->n[0], n1 = bp->n[1], n2 = bp->n[2];
   const float ix = bp->fidx2[0], iy = bp->fidx2[1], iz = bp->fidx2[2], j0 = bp->fj0;
   const CUtensorMap *me = maps + MT_NMAPS * tl.box + (src == W_E2 ? 1 : 0), *md = maps + MT_NMAPS * tl.box + 2,
                     *mc = maps + MT_NMAPS * tl.box + 3;
   const int i0 = tl.i0, jb = tl.j0, kb = tl.k0, ke = min(tl.k0 + lv.mtz, n2);   /* planes [kb, ke) written */
   if (kb & 1) {   /* the unrolled colours assume an even first plane */
      if (threadIdx.x == 0) *err = 2;
      return;
   }
   const int t = threadIdx.x, w = t >> 5;
   const int tx = (w % S::HX) * 16 + (t & 15), ty = 2 * (w / S::HX) + ((t >> 4) & 1);
   const int gy = jb - 3 + ty, xs = i0 - 4 + 2 * tx + (gy & 1);   /* the pair: (xs, xs+1) of row gy, xs + gy even */
   float *const s0 = sm + (1 + ty) * EW + 2 * tx + (gy & 1);      /* the first member in slot 0's E plane */
   const bool yin = gy >= 1 && gy <= n1 - 2;
   const bool xin0 = yin && xs >= 1 && xs <= n0 - 2, xin1 = yin && xs >= 0 && xs <= n0 - 3;
   /* the column grown by h points holds member x */
   auto grown = [&](int x, int h) {
      return x >= i0 - h && x <= i0 + TXO - 1 + h && gy >= jb - h && gy <= jb + MT_TYO - 1 + h;
   };
   const bool g3_0 = grown(xs, 3), g3_1 = grown(xs + 1, 3), g2_0 = grown(xs, 2), g2_1 = grown(xs + 1, 2);
   const bool g1_0 = grown(xs, 1), g1_1 = grown(xs + 1, 1);
   const bool out0 = grown(xs, 0) && xs < n0 && gy < n1, out1 = grown(xs + 1, 0) && xs + 1 < n0 && gy < n1;
   float *gp = bp->w32[dst] + (out0 || out1 ? xs + bp->wy * gy : 0);
   const long wz = bp->wz;
   if (t == 0) {
      for (int r = 0; r < MT_R; r++)
         asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mt_saddr(bar + r)), "r"(1) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
   }
   __syncthreads();
   const int m0 = kb - 4, mlast = min(ke + 3, n2 - 1);
   int last_issued = m0 - 1;
   auto issue = [&](int m) {   /* thread 0 */
      uint64_t *b = bar + ((m - m0) & (MT_R - 1));
      last_issued = m;
      if (m < 0 || m > mlast) {
         asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mt_saddr(b)) : "memory");
         return;
      }
      float *sl = sm + ((m - m0) & (MT_R - 1)) * SL;
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mt_saddr(b)),
                   "r"(S::EBYTES + 2 * S::DBYTES) : "memory");
      mt_load(sl, me, i0 - 4, jb - 4, m, b);
      mt_load(sl + S::ESZ, md, i0 - 4, jb - 3, m, b);
      mt_load(sl + S::ESZ + S::DSZ, mc, i0 - 4, jb - 3, m, b);
   };
   if (t == 0)
      for (int m = m0; m < m0 + MT_R; m++) issue(m);
   bool ok = true;
   int waited = m0 - 1;
   for (int q = m0; q <= min(kb - 3, mlast); q++) {   /* planes kb-4, kb-3 (slots 0, 1) */
      if (q >= 0 && !mt_wait(bar + (q - m0), 0)) ok = false;
      waited = q;
   }
   float zprev = s0[SL + 1], aprev = s0[0];
   float rp1 = 0.f, rp2 = 0.f;   /* first sweep, first colour: (other member, k-1), (c, k-2) */
   float b0 = 0.f, b1 = 0.f;     /* first sweep, second colour: (other member, k-2), (c, k-3) */
   float q1 = 0.f, q2 = 0.f;     /* second sweep, first colour: (other member, k-3), (c, k-4) */
   gp += wz * (long)(kb - 7);   /* advanced to plane k-3 at each step */

   /* step s: plane k = kb - 3 + s, slot (s + 1) % R; colour member mem = s % 2 */
   for (int sb = 0;; sb += MT_R) {
      const uint32_t ph = (sb / MT_R) & 1;
#pragma unroll
      for (int u = 0; u < MT_R; u++) {
         const int s = sb + u, k = kb - 3 + s;
         if (k > ke + 2) return;
         const int mem = u & 1;
         const int jk = ((u + 1) & (MT_R - 1)) * SL, jm = (u & (MT_R - 1)) * SL, jp = ((u + 2) & (MT_R - 1)) * SL;
         const int jm2 = ((u + MT_R - 1) & (MT_R - 1)) * SL, jm3 = ((u + MT_R - 2) & (MT_R - 1)) * SL;
         if (k + 1 <= mlast) {
            if (!mt_wait(bar + ((u + 2) & (MT_R - 1)), ph ^ (u + 2 >= MT_R ? 1u : 0u))) ok = false;
            waited = k + 1;
         }
         float *pc = s0 + mem;
         const bool xin = mem ? xin1 : xin0;
         /* first sweep, first colour at (c, k) */
         const float ec = pc[jk], ea = zprev, ezm = aprev;
         const float eb = mem ? pc[jk + 1] : pc[jk - 1];
         const float zp = pc[jp];
         float rk = gs32(ec, mem ? ea : eb, mem ? eb : ea, pc[jk - EW], pc[jk + EW], ezm, zp, pc[jk + CO],
                         pc[jk + DO], ix, iy, iz, j0, true);
         if (!(xin && k >= 1 && k <= n2 - 2)) rk = ec;
         if (mem ? g3_1 : g3_0) pc[jk] = rk;
         /* first sweep, second colour at (c, k-1), kept in its slot */
         float bk = ezm;
         if (s >= 2) {
            const float fb = mem ? pc[jm + 1] : pc[jm - 1];
            bk = gs32(ezm, mem ? rp1 : fb, mem ? fb : rp1, pc[jm - EW], pc[jm + EW], rp2, rk, pc[jm + CO], pc[jm + DO],
                      ix, iy, iz, j0, true);
            if (!(xin && k >= 2 && k <= n2 - 1)) bk = ezm;
            if (mem ? g2_1 : g2_0) pc[jm] = bk;
         }
         /* second sweep, first colour at (c, k-2) */
         float q = 0.f;
         gp += wz;
         if (s >= 4) {
            const float old = pc[jm2];
            const float fb2 = mem ? pc[jm2 + 1] : pc[jm2 - 1];
            q = gs32(old, mem ? b0 : fb2, mem ? fb2 : b0, pc[jm2 - EW], pc[jm2 + EW], b1, bk, pc[jm2 + CO],
                     pc[jm2 + DO], ix, iy, iz, j0, true);
            if (!(xin && k >= 3 && k <= n2)) q = old;
            if (mem ? g1_1 : g1_0) pc[jm2] = q;
         }
         /* second sweep, second colour at (c, k-3); plane k-3 is final */
         if (s >= 6 && k - 3 < ke) {
            const float fb3 = mem ? pc[jm3 + 1] : pc[jm3 - 1];
            float b2 = gs32(b1, mem ? q1 : fb3, mem ? fb3 : q1, pc[jm3 - EW], pc[jm3 + EW], q2, q, pc[jm3 + CO],
                            pc[jm3 + DO], ix, iy, iz, j0, true);
            if (!(xin && k >= 4 && k <= n2 + 1)) b2 = b1;
            if (out0) gp[0] = mem ? q1 : b2;
            if (out1) gp[1] = mem ? b2 : q1;
         }
         zprev = zp;
         aprev = ea;
         rp2 = rp1;
         rp1 = rk;
         b1 = b0;
         b0 = bk;
         q2 = q1;
         q1 = q;
         if (!ok) *err = 1;
         if (__syncthreads_or(!ok)) {   /* a load never landed: let the issued ones land, return */
            if (t == 0)
               for (int qq = max(waited + 1, 0); qq <= min(mlast, last_issued); qq++)
                  mt_wait(bar + ((qq - m0) & (MT_R - 1)), ((qq - m0) / MT_R) & 1);
            return;
         }
         /* plane k-3's slot is free: every thread is past step k */
         if (t == 0 && s >= 2) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(k - 3 + MT_R);
         }
      }
   }
}

/* Tensor maps of the TMA sweeps: per box, for the column widths 60 and 28
 * (one sweep per launch) and 24 and 56 (two), the old correction in slot 0
 * and slot 4, D and C (3-D tiles of the padded FP32 arrays; out-of-box
 * coordinates read as zero). */
#include <cudaTypedefs.h>

static int mt_encode(PFN_cuTensorMapEncodeTiled_v12000 enc, CUtensorMap *m, const float *base, const pgb_dbox &b,
                     int w, int h)
{
   cuuint64_t dims[3] = {(cuuint64_t)b.n[0], (cuuint64_t)b.n[1], (cuuint64_t)b.n[2]};
   cuuint64_t strides[2] = {(cuuint64_t)b.wy * 4, (cuuint64_t)b.wz * 4};
   cuuint32_t box[3] = {(cuuint32_t)w, (cuuint32_t)h, 1}, es[3] = {1, 1, 1};
   CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void *)base, dims, strides, box, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
   return r != CUDA_SUCCESS;
}

/* builds MT_NMAPS maps per box (widths 60, 28, 24, 56 x slot 0, slot 4, D, C) in device
 * memory; returns 0, or 1 when the driver has no tensor-map encoder or a
 * box is not 3-D (the TMA sweep is then not offered) */
extern "C" int pgb_tmaps_build(const pgb_dbox *hbox, int nbox, void **d_maps)
{
   static PFN_cuTensorMapEncodeTiled_v12000 enc = 0;
   *d_maps = 0;
   if (!enc) {
      cudaDriverEntryPointQueryResult q;
      void *fn = 0;
      if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
              cudaSuccess ||
          q != cudaDriverEntryPointSuccess || !fn) {
         cudaGetLastError();
         return 1;
      }
      enc = (PFN_cuTensorMapEncodeTiled_v12000)fn;
   }
   CUtensorMap *h = (CUtensorMap *)calloc((size_t)nbox * MT_NMAPS, sizeof(CUtensorMap));
   int bad = 0;
   for (int i = 0; i < nbox && !bad; i++) {
      const pgb_dbox &b = hbox[i];
      if (b.n[2] < 3 || !b.w32[W_E]) {
         bad = 1;
         break;
      }
      /* E grown by 2 rows (one sweep) or 4 (two), D and C by 1 or 3 */
      const int txo[4] = {60, 28, 24, 56}, grow[4] = {2, 2, 4, 4};
      for (int v = 0; v < 4 && !bad; v++) {
         CUtensorMap *m = h + MT_NMAPS * i + 4 * v;
         const int w = txo[v] + 8;
         bad |= mt_encode(enc, m + 0, b.w32[W_E], b, w, MT_TYO + 2 * grow[v]);
         bad |= mt_encode(enc, m + 1, b.w32[W_E2], b, w, MT_TYO + 2 * grow[v]);
         bad |= mt_encode(enc, m + 2, b.w32[W_D], b, w, MT_TYO + 2 * grow[v] - 2);
         bad |= mt_encode(enc, m + 3, b.w32[W_C], b, w, MT_TYO + 2 * grow[v] - 2);
      }
   }
   if (!bad && cudaMalloc(d_maps, sizeof(CUtensorMap) * MT_NMAPS * (size_t)nbox) == cudaSuccess)
      bad = cudaMemcpy(*d_maps, h, sizeof(CUtensorMap) * MT_NMAPS * (size_t)nbox, cudaMemcpyHostToDevice) != cudaSuccess;
   else
      bad = 1;
   free(h);
   if (bad) {
      if (*d_maps) cudaFree(*d_maps);
      *d_maps = 0;
      cudaGetLastError();
      return 1;
   }
   return 0;
}

/* one TMA sweep of level lv from slot src into slot dst (two with the
 * column widths 24 and 56); maps from pgb_tmaps_build, lv.mtx the column
 * width the level's tile list was made for */
static int sweep32t(const pgb_dbox *boxes, pgb_dlevel lv, const void *maps, int src, int dst, int *err,
                    cudaStream_t st)
{
   if (!lv.nmtiles) return 0;
   static int attr = 0;
   if (!attr) {
      cudaFuncSetAttribute(k_sweep32t<60>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mt_shape<60>::SMEM);
      cudaFuncSetAttribute(k_sweep32t<28>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mt_shape<28>::SMEM);
      cudaFuncSetAttribute(k_sweep32t2<24>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mt2_shape<24>::SMEM);
      cudaFuncSetAttribute(k_sweep32t2<56>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mt2_shape<56>::SMEM);
      attr = 1;
   }
   /* per box, the maps of width 60 sit at MT_NMAPS i + 0..3, 28 at 4..7, 24 at 8..11, 56 at 12..15 */
   const CUtensorMap *m = (const CUtensorMap *)maps;
   if (lv.mtx == 60)
      k_sweep32t<60><<<lv.nmtiles, mt_shape<60>::NTH, mt_shape<60>::SMEM, st>>>(boxes, lv, m, src, dst, err);
   else if (lv.mtx == 28)
      k_sweep32t<28><<<lv.nmtiles, mt_shape<28>::NTH, mt_shape<28>::SMEM, st>>>(boxes, lv, m + 4, src, dst, err);
   else if (lv.mtx == 24)
      k_sweep32t2<24><<<lv.nmtiles, mt2_shape<24>::NTH, mt2_shape<24>::SMEM, st>>>(boxes, lv, m + 8, src, dst, err);
   else
      k_sweep32t2<56><<<lv.nmtiles, mt2_shape<56>::NTH, mt2_shape<56>::SMEM, st>>>(boxes, lv, m + 12, src, dst, err);
   return check32("sweep32t");
}

/* E = the correction in slot src, over the level's tiles (the end of an
 * odd number of fused sweep launches) */
template <bool TAIL>
__device__ __forceinline__ void copy_e_b(const vblk &vb, const pgb_dbox *boxes, const pgb_dlevel &lv, int src)
{
   const pgb_tile tl = lv.tiles[vb.x];
   const pgb_dbox b = boxes[tl.box];
   const int i = tl.i0 + threadIdx.x, j = tl.j0 + threadIdx.y;
   if (i >= b.n[0] || j >= b.n[1]) return;
   const int kz = lv.dim == 3 ? lv.tz : 1;
   RP(const float) a = eslot(b, src);
   RP(float) e = b.w32[W_E];
   for (int kk = 0; kk < kz; kk++) {
      const int k = tl.k0 + kk;
      if (k >= b.n[2]) break;
      const long q = wq(b, i, j, k);
      e[q] = a[q];
   }
}

__global__ void __launch_bounds__(NT) k_copy_e(const pgb_dbox *boxes, pgb_dlevel lv, int src)
{
   copy_e_b<false>(hw_blk(), boxes, lv, src);
}

/* D = D - (lap E + C E) at the relaxed points, FP32, before the update that
 * adds E to u: the defect of u + E, linearised, for the next cycle's
 * pre-smoothing on a level whose points outside the cover tiles do not
 * change in between (no sync, no injection there). The next FP64 residual
 * (after that pre-smoothing) is computed from u itself. */
/* D - (lap E + C E) at point q of E (rows of pitch wy, planes wz): the one
 * expression of the FP32 defect carry, shared by k_defect32 and
 * k_update_defect so that both round alike */
__device__ __forceinline__ float defect32_at(const float *e, long q, long wy, long wz, float c,
                                             float d, float ix, float iy, float iz, int dim)
{
   const float ec = e[q];
   float t = (e[q + 1] - 2.f * ec + e[q - 1]) * ix + (e[q + wy] - 2.f * ec + e[q - wy]) * iy;
   if (dim == 3) t += (e[q + wz] - 2.f * ec + e[q - wz]) * iz;
   return d - (t + c * ec);
}

template <bool TAIL>
__device__ __forceinline__ void defect32_b(const vblk &vb, const pgb_dbox *boxes, const pgb_dlevel &lv, int slot,
                                           int split, const int *gate, int gval)
{
   if (gate && *gate != gval) return;   /* the cycle parity leaves this pass out */
   const tile_part tp = tile_split(lv.tiles, lv, split, vb.x);
   const pgb_tile tl = tp.tl;
   const pgb_dbox b = boxes[tl.box];
   const int dim = lv.dim;
   const int i = tl.i0 + threadIdx.x, j = tl.j0 + threadIdx.y;
   if (i >= b.n[0] || j >= b.n[1]) return;
   RP(const float) e = eslot(b, slot);
   RP(const float) cc = b.w32[W_C];
   RP(float) dd = b.w32[W_D];
   const long sy = b.n[0], sz = (long)b.n[0] * b.n[1];
   const float ix = b.fidx2[0], iy = b.fidx2[1], iz = b.fidx2[2];
#pragma unroll
   for (int kk = 0; kk < PGB_TZ; kk++) {
      const int k = tl.k0 + tp.kk0 + kk;
      if (kk >= tp.nk || k >= b.n[2]) continue;
      const long p = i + sy * j + sz * k, q = wq(b, i, j, k);
      if (!relaxed32(b, i, j, k, p, dim)) continue;
      dd[q] = defect32_at(e, q, b.wy, b.wz, cc[q], dd[q], ix, iy, iz, dim);
   }
}

__global__ void __launch_bounds__(NT) k_defect32(const pgb_dbox *boxes, pgb_dlevel lv, int slot, int split,
                                                 const int *gate, int gval)
{
   defect32_b<false>(hw_blk(), boxes, lv, slot, split, gate, gval);
}

/* End of a smoothing block: u += E (FP64, E from the slot the sweeps
 * ended in) and E = 0 in slot zslot, where the next block starts (the same
 * slot costs no extra traffic). After an
 * interpolated coarse-grid correction (post = 1) the points the smoother
 * does not relax take the FP64 correction the interpolation left in res,
 * plus whatever a sync of E brought in: u += res + (E - d2f(res)), exactly
 * res when E still holds the d2f(res) the interpolation wrote (the fused
 * sweeps copy unrelaxed points from slot to slot). */
template <bool TAIL>
__device__ __forceinline__ void update_b(const vblk &vb, const pgb_dbox *boxes, const pgb_dlevel &lv, int post,
                                         int slot, int zslot, int split)
{
   const tile_part tp = tile_split(lv.tiles, lv, split, vb.x);
   const pgb_tile tl = tp.tl;
   const pgb_dbox b = boxes[tl.box];
   const int i = tl.i0 + threadIdx.x, j = tl.j0 + threadIdx.y;
   if (i >= b.n[0] || j >= b.n[1]) return;
   RP(double) u = b.f[PGB_F_U];
   const float *es = eslot(b, slot);
   float *e = eslot(b, zslot);
   RP(const double) res = b.f[PGB_F_RES];
#pragma unroll
   for (int kk = 0; kk < PGB_TZ; kk++) {
      const int k = tl.k0 + tp.kk0 + kk;
      if (kk >= tp.nk || k >= b.n[2]) continue;
      const long p = i + (long)b.n[0] * (j + (long)b.n[1] * k), q = wq(b, i, j, k);
      double corr = f2d(es[q]);
      if (post && !relaxed32(b, i, j, k, p, lv.dim)) {
         const double r = res[p];
         corr += r - f2d(d2f(r));
      }
      u[p] += corr;
      e[q] = 0.f;
   }
}

__global__ void __launch_bounds__(NT) k_update(const pgb_dbox *boxes, pgb_dlevel lv, int post, int slot,
                                               int zslot, int split)
{
   update_b<false>(hw_blk(), boxes, lv, post, slot, zslot, split);
}

/* k_defect32 and k_update in one pass, for blocks whose update zeroes the
 * other slot (zslot != slot): the defect reads E's stencil in slot while
 * the update writes zeros only to zslot. The defect part runs unless the
 * cycle parity gate leaves it out (gate && *gate != gval); with defect = 0
 * this is k_update. Same arithmetic as the two kernels. */
template <bool TAIL>
__device__ __forceinline__ void update_defect_b(const vblk &vb, const pgb_dbox *boxes, const pgb_dlevel &lv, int post,
                                                int slot, int zslot, int split, int defect, const int *gate, int gval)
{
   const tile_part tp = tile_split(lv.tiles, lv, split, vb.x);
   const pgb_tile tl = tp.tl;
   const pgb_dbox b = boxes[tl.box];
   const int i = tl.i0 + threadIdx.x, j = tl.j0 + threadIdx.y;
   if (i >= b.n[0] || j >= b.n[1]) return;
   const bool dfx = defect && (!gate || *gate == gval);
   RP(double) u = b.f[PGB_F_U];
   RP(const float) es = eslot(b, slot);
   RP(float) ez = eslot(b, zslot);
   RP(const double) res = b.f[PGB_F_RES];
   RP(const float) cc = b.w32[W_C];
   RP(float) dd = b.w32[W_D];
   const float ix = b.fidx2[0], iy = b.fidx2[1], iz = b.fidx2[2];
#pragma unroll
   for (int kk = 0; kk < PGB_TZ; kk++) {
      const int k = tl.k0 + tp.kk0 + kk;
      if (kk >= tp.nk || k >= b.n[2]) continue;
      const long p = i + (long)b.n[0] * (j + (long)b.n[1] * k), q = wq(b, i, j, k);
      const bool rel = relaxed32(b, i, j, k, p, lv.dim);
      if (dfx && rel) dd[q] = defect32_at(es, q, b.wy, b.wz, cc[q], dd[q], ix, iy, iz, lv.dim);
      double corr = f2d(es[q]);
      if (post && !rel) {
         const double r = res[p];
         corr += r - f2d(d2f(r));
      }
      u[p] += corr;
      ez[q] = 0.f;
   }
}

__global__ void __launch_bounds__(NT) k_update_defect(const pgb_dbox *boxes, pgb_dlevel lv, int post, int slot,
                                                      int zslot, int split, int defect, const int *gate, int gval)
{
   update_defect_b<false>(hw_blk(), boxes, lv, post, slot, zslot, split, defect, gate, gval);
}

/* zero the four FP32 arrays (pgb_prepare) */
__global__ void __launch_bounds__(NT) k_zero32(const pgb_dbox *boxes, pgb_dlevel lv)
{
   const pgb_tile tl = lv.tiles[blockIdx.x];
   const pgb_dbox b = boxes[tl.box];
   const int i = tl.i0 + threadIdx.x, j = tl.j0 + threadIdx.y;
   if (i >= b.n[0] || j >= b.n[1]) return;
   const int kz = lv.dim == 3 ? lv.tz : 1;
#pragma unroll
   for (int kk = 0; kk < PGB_TZ; kk++) {
      const int k = tl.k0 + kk;
      if (kk >= kz || k >= b.n[2]) continue;
      const long q = wq(b, i, j, k);
      for (int f = 0; f < 4; f++) b.w32[f][q] = 0.f;
   }
}

__device__ __forceinline__ long lin32(const pgb_dbox &b, int i1, int j1, int k1)
{
   return (i1 - 1) + (long)b.n[0] * ((j1 - 1) + (long)b.n[1] * (k1 - 1));
}

/* the same 1-based point in the box's FP32 arrays */
__device__ __forceinline__ long lin32w(const pgb_dbox &b, int i1, int j1, int k1)
{
   return wq(b, i1 - 1, j1 - 1, k1 - 1);
}

/* FP32 copy of the correction in slot `slot` along a sync plan (PAMR_sync
 * of E) */
__global__ void k_copy32(const pgb_dbox *boxes, const pgb_copy_op *ops, int slot)
{
   const pgb_copy_op o = ops[blockIdx.z];
   const pgb_dbox &s = boxes[o.src_box];
   const pgb_dbox &d = boxes[o.dst_box];
   OP_PLANES(o.ni, o.nj, o.nk, {
      eslot(d, slot)[lin32w(d, o.i2 + a, o.j2 + bb, o.k2 + c)] =
         eslot(s, slot)[lin32w(s, o.i1 + a, o.j1 + bb, o.k1 + c)];
   })
}

/* window stencil of dminterp3d (src/m_util_r8.f:65-144) in FP32: linear, or
 * cubic with one-sided ends; n = 1 marks a copied anchor */
__device__ __forceinline__ int stencil32(int t, int irho, int nanch, int ord, int *a, float *cf)
{
   const int m = irho == 2 ? t >> 1 : t / irho, j = t - m * irho;
   if (j == 0) {
      a[0] = m;
      return 1;
   }
   if (ord == 2 || nanch < 4) {
      const float sg = (irho == 2 ? (float)j * 0.5f : (float)j / irho);
      cf[0] = 1.f - sg;
      cf[1] = sg;
      a[0] = m;
      a[1] = m + 1;
      return 2;
   }
   float sg;
   int base;
   if (m == 0) {
      sg = (irho == 2 ? (float)j * 0.5f : (float)j / irho);
      base = 0;
   } else if (m == nanch - 2) {
      sg = 2.f + (irho == 2 ? (float)j * 0.5f : (float)j / irho);
      base = nanch - 4;
   } else {
      sg = 1.f + (irho == 2 ? (float)j * 0.5f : (float)j / irho);
      base = m - 1;
   }
   cf[0] = -(1.f / 6.f) * (sg - 1.f) * (sg - 2.f) * (sg - 3.f);
   cf[1] = 0.5f * sg * (sg - 2.f) * (sg - 3.f);
   cf[2] = -0.5f * sg * (sg - 1.f) * (sg - 3.f);
   cf[3] = (1.f / 6.f) * sg * (sg - 1.f) * (sg - 2.f);
   for (int q = 0; q < 4; q++) a[q] = base + q;
   return 4;
}

__device__ __forceinline__ float wsum32(int n, const float *c, const float *v)
{
   if (n == 1) return v[0];
   float r = c[0] * v[0] + c[1] * v[1];
   if (n == 4) r = r + c[2] * v[2] + c[3] * v[3];
   return r;
}

/* the same window stencil with FP64 weights */
__device__ __forceinline__ int stencil64m(int t, int irho, int nanch, int ord, int *a, double *cf)
{
   const int m = irho == 2 ? t >> 1 : t / irho, j = t - m * irho;
   if (j == 0) {
      a[0] = m;
      return 1;
   }
   if (ord == 2 || nanch < 4) {
      const double sg = (irho == 2 ? (double)j * 0.5 : (double)j / irho);
      cf[0] = 1.0 - sg;
      cf[1] = sg;
      a[0] = m;
      a[1] = m + 1;
      return 2;
   }
   double sg;
   int base;
   if (m == 0) {
      sg = (irho == 2 ? (double)j * 0.5 : (double)j / irho);
      base = 0;
   } else if (m == nanch - 2) {
      sg = 2.0 + (irho == 2 ? (double)j * 0.5 : (double)j / irho);
      base = nanch - 4;
   } else {
      sg = 1.0 + (irho == 2 ? (double)j * 0.5 : (double)j / irho);
      base = m - 1;
   }
   cf[0] = -(1.0 / 6.0) * (sg - 1.0) * (sg - 2.0) * (sg - 3.0);
   cf[1] = 0.5 * sg * (sg - 2.0) * (sg - 3.0);
   cf[2] = -0.5 * sg * (sg - 1.0) * (sg - 3.0);
   cf[3] = (1.0 / 6.0) * sg * (sg - 1.0) * (sg - 2.0);
   for (int q = 0; q < 4; q++) a[q] = base + q;
   return 4;
}

__device__ __forceinline__ double wsum64m(int n, const double *c, const double *v)
{
   if (n == 1) return v[0];
   double r = c[0] * v[0] + c[1] * v[1];
   if (n == 4) r = r + c[2] * v[2] + c[3] * v[3];
   return r;
}

/* Coarse half of the coarse-grid correction (amrd/mg.c:332-341) on the tiles
 * the interpolation reads: res = (f - lop)/w0_i in FP64, X = RN32(res). */
__device__ __forceinline__ void cgc_mixed_b(const vblk &vb, const pgb_dbox *boxes, const pgb_dlevel &lv,
                                            double inv_w0, int split)
{
   const tile_part tp = tile_split(lv.ctiles, lv, split, vb.x);
   const pgb_tile tl = tp.tl;
   const pgb_dbox b = boxes[tl.box];
   const int i = tl.i0 + threadIdx.x, j = tl.j0 + threadIdx.y;
   if (i >= b.n[0] || j >= b.n[1]) return;
#pragma unroll
   for (int kk = 0; kk < PGB_TZ; kk++) {
      const int k = tl.k0 + tp.kk0 + kk;
      if (kk >= tp.nk || k >= b.n[2]) continue;
      const long p = i + (long)b.n[0] * (j + (long)b.n[1] * k);
      const double r = (b.f[PGB_F_U][p] - b.f[PGB_F_LOP][p]) * inv_w0;
      b.f[PGB_F_RES][p] = r;
      b.w32[W_X][wq(b, i, j, k)] = d2f(r);
   }
}

__global__ void __launch_bounds__(NT) k_cgc_mixed(const pgb_dbox *boxes, pgb_dlevel lv, double inv_w0,
                                                  int split)
{
   cgc_mixed_b(hw_blk(), boxes, lv, inv_w0, split);
}

/* FP64 interpolation of the coarse res at window point (a, bb, c) of op o
 * (dminterp3d's line order: i, then j, then k) */
template <bool TAIL>
__device__ __noinline__ double interp_point64(const pgb_interp_op &o, const pgb_dbox &s, int a, int bb, int c, int dim)
{
   RP(const double) u = s.f[PGB_F_RES];
   int ax[4], ay[4], az[4];
   double cx[4], cy[4], cz[4], kv[4];
   const int nx = stencil64m(o.i2b - 1 + a, o.irho, o.nii, o.ord, ax, cx);
   const int ny = stencil64m(o.j2b - 1 + bb, o.irho, o.nji, o.ord, ay, cy);
   const int nz = dim == 3 ? stencil64m(o.k2b - 1 + c, o.irho, o.nki, o.ord, az, cz) : 1;
   if (dim != 3) az[0] = 0;
   for (int r = 0; r < nz; r++) {
      double jv[4];
      for (int qq = 0; qq < ny; qq++) {
         double iv[4];
         for (int pp = 0; pp < nx; pp++) iv[pp] = u[lin32(s, o.i1i + ax[pp], o.j1i + ay[qq], o.k1i + az[r])];
         jv[qq] = wsum64m(nx, cx, iv);
      }
      kv[r] = wsum64m(ny, cy, jv);
   }
   return wsum64m(nz, cz, kv);
}

/* Fine half (amrd/mg.c:343-354), PAMR_interp in plan order (ops of one
 * batch write disjoint points, later batches overwrite earlier ones like the
 * reference's sequential transfers). Relaxed points: E = interpolation of X
 * in FP32, the start of the post-smoothing block. Other points: the FP64
 * interpolation of the coarse res into res (k_update adds it) and its FP32
 * value into E, which the smoother reads as a neighbour. FP64 issues at a
 * small fraction of the FP32 rate, so FP64 points are kept in dense warps:
 * on boxes whose interior is all relaxed this kernel leaves the face rows
 * and the two x-ends of the other rows to k_interp_edges. */
template <bool TAIL>
__device__ __forceinline__ void interp_mixed_b(const vblk &vb, const pgb_dbox *boxes, const pgb_interp_op *ops, int dim,
                                               int slot)
{
   const pgb_interp_op o = ops[vb.z];
   const pgb_dbox &s = boxes[o.src_box];
   const pgb_dbox &d = boxes[o.dst_box];
   const bool allrel = d.flags & PGB_BOX_BDY_INTERIOR;
   RP(const float) x = s.w32[W_X];
   for (int row = vb.y; row < o.njb * o.nkb; row += vb.gy) {
      const int bb = row % o.njb, c = row / o.njb;
      const int fj = o.j2 + bb, fk = o.k2 + c;
      const bool face = fj == 1 || fj == d.n[1] || (dim == 3 && (fk == 1 || fk == d.n[2]));
      int ay[4], az[4];
      float cy[4], cz[4];
      const int ny = stencil32(o.j2b - 1 + bb, o.irho, o.nji, o.ord, ay, cy);
      const int nz = dim == 3 ? stencil32(o.k2b - 1 + c, o.irho, o.nki, o.ord, az, cz) : 1;
      if (dim != 3) az[0] = 0;
      for (int a = vb.x * vb.nt + vb.lt; a < o.nib; a += vb.gx * vb.nt) {
         const int fi = o.i2 + a;
         const long pd = lin32(d, fi, fj, fk), pw = lin32w(d, fi, fj, fk);
         bool fp64;
         if (allrel) {
            if (face || fi == 1 || fi == d.n[0]) continue;   /* k_interp_edges */
            fp64 = false;
         } else
            fp64 = !relaxed32(d, fi - 1, fj - 1, fk - 1, pd, dim);
         if (fp64) {
            const double v = interp_point64<TAIL>(o, s, a, bb, c, dim);
            d.f[PGB_F_RES][pd] = v;
            eslot(d, slot)[pw] = d2f(v);
            continue;
         }
         int ax[4];
         float cx[4], kv[4];
         const int nx = stencil32(o.i2b - 1 + a, o.irho, o.nii, o.ord, ax, cx);
         for (int r = 0; r < nz; r++) {
            float jv[4];
            for (int qq = 0; qq < ny; qq++) {
               float iv[4];
               for (int pp = 0; pp < nx; pp++) iv[pp] = x[lin32w(s, o.i1i + ax[pp], o.j1i + ay[qq], o.k1i + az[r])];
               jv[qq] = wsum32(nx, cx, iv);
            }
            kv[r] = wsum32(ny, cy, jv);
         }
         eslot(d, slot)[pw] = wsum32(nz, cz, kv);
      }
   }
}

__global__ void k_interp_mixed(const pgb_dbox *boxes, const pgb_interp_op *ops, int dim, int slot)
{
   interp_mixed_b<false>(hw_blk(), boxes, ops, dim, slot);
}

/* k_interp_mixed for ops of ratio 2 and linear order (every MG hierarchy
 * with the default interpolation): the FP32 value of a fine point is the mean
 * of its (up to 8 distinct) coarse corners, counted with multiplicity. */
template <bool TAIL>
__device__ __forceinline__ void interp_lin2_b(const vblk &vb, const pgb_dbox *boxes, const pgb_interp_op *ops, int dim,
                                              int slot)
{
   const pgb_interp_op o = ops[vb.z];
   const pgb_dbox &s = boxes[o.src_box];
   const pgb_dbox &d = boxes[o.dst_box];
   const bool allrel = d.flags & PGB_BOX_BDY_INTERIOR;
   RP(const float) x = s.w32[W_X];
   RP(float) e = eslot(d, slot);
   RP(double) res = d.f[PGB_F_RES];
   const long sny = s.n[0], snz = (long)s.n[0] * s.n[1];
   const long dny = d.n[0], dnz = (long)d.n[0] * d.n[1];
   const long swy = s.wy, swz = s.wz, dwy = d.wy, dwz = d.wz;   /* FP32 pitches */
   for (int row = vb.y; row < o.njb * o.nkb; row += vb.gy) {
      const int bb = row % o.njb, c = row / o.njb;
      const int fj = o.j2 + bb, fk = o.k2 + c;
      const bool face = fj == 1 || fj == d.n[1] || (dim == 3 && (fk == 1 || fk == d.n[2]));
      if (allrel && face) continue;
      const int ty = o.j2b - 1 + bb, tz = dim == 3 ? o.k2b - 1 + c : 0;
      const long oy = (ty & 1) ? sny : 0, oz = (tz & 1) ? snz : 0;
      const long rowc = (o.j1i - 1 + (ty >> 1)) * sny + (dim == 3 ? (o.k1i - 1 + (tz >> 1)) * snz : 0);
      const long rowf = (long)(fj - 1) * dny + (long)(fk - 1) * dnz;
      const long oyw = (ty & 1) ? swy : 0, ozw = (tz & 1) ? swz : 0;
      const long rowcw = (o.j1i - 1 + (ty >> 1)) * swy + (dim == 3 ? (o.k1i - 1 + (tz >> 1)) * swz : 0);
      const long rowfw = (long)(fj - 1) * dwy + (long)(fk - 1) * dwz;
      for (int a = vb.x * vb.nt + vb.lt; a < o.nib; a += vb.gx * vb.nt) {
         const int fi = o.i2 + a;
         const long pd = rowf + fi - 1, pw = rowfw + fi - 1;
         const int tx = o.i2b - 1 + a, ox = tx & 1;
         if (allrel) {
            if (face || fi == 1 || fi == d.n[0]) continue;   /* k_interp_edges */
         } else if (!relaxed32(d, fi - 1, fj - 1, fk - 1, pd, dim)) {
            const double *c0 = s.f[PGB_F_RES] + rowc + (o.i1i - 1 + (tx >> 1));
            const double v = 0.125 * (((c0[0] + c0[ox]) + (c0[oy] + c0[ox + oy])) +
                                      ((c0[oz] + c0[ox + oz]) + (c0[oy + oz] + c0[ox + oy + oz])));
            res[pd] = v;
            e[pw] = d2f(v);
            continue;
         }
         const float *c0 = x + rowcw + (o.i1i - 1 + (tx >> 1));
         const float v = ((c0[0] + c0[ox]) + (c0[oyw] + c0[ox + oyw])) +
                         ((c0[ozw] + c0[ox + ozw]) + (c0[oyw + ozw] + c0[ox + oyw + ozw]));
         e[pw] = 0.125f * v;
      }
   }
}

__global__ void __launch_bounds__(128, 8) k_interp_lin2(const pgb_dbox *boxes, const pgb_interp_op *ops, int dim,
                                                         int slot)
{
   interp_lin2_b<false>(hw_blk(), boxes, ops, dim, slot);
}

/* The FP64 points of ops into boxes whose interior is all relaxed: the rows
 * on a box face (j or k at the box boundary), blockIdx.y < 2*(njb+nkb)
 * picking the face and the row on it, and, for the remaining blockIdx.y,
 * the two x-ends (fi = 1, n) of the other rows, one per thread. */
template <bool TAIL>
__device__ __forceinline__ void interp_edges_b(const vblk &vb, const pgb_interp_op *ops, const pgb_dbox *boxes, int dim,
                                               int slot)
{
   const pgb_interp_op o = ops[vb.z];
   const pgb_dbox &s = boxes[o.src_box];
   const pgb_dbox &d = boxes[o.dst_box];
   if (!(d.flags & PGB_BOX_BDY_INTERIOR)) return;
   const int y = vb.y, nface = 2 * (o.njb + o.nkb);
   if (y < nface) {
      int bb, c;
      if (y < 2 * o.nkb) {
         bb = ((y / o.nkb) ? d.n[1] : 1) - o.j2;
         c = y % o.nkb;
      } else {
         if (dim != 3) return;
         const int y2 = y - 2 * o.nkb;
         c = ((y2 / o.njb) ? d.n[2] : 1) - o.k2;
         bb = y2 % o.njb;
         const int fj = o.j2 + bb;
         if (fj == 1 || fj == d.n[1]) return;   /* done as a j face */
      }
      if (bb < 0 || bb >= o.njb || c < 0 || c >= o.nkb) return;
      const int fj = o.j2 + bb, fk = o.k2 + c;
      for (int a = vb.x * vb.nt + vb.lt; a < o.nib; a += vb.gx * vb.nt) {
         const long pd = lin32(d, o.i2 + a, fj, fk);
         const double v = interp_point64<TAIL>(o, s, a, bb, c, dim);
         d.f[PGB_F_RES][pd] = v;
         eslot(d, slot)[lin32w(d, o.i2 + a, fj, fk)] = d2f(v);
      }
      return;
   }
   if (vb.x) return;
   const int rows = o.njb * o.nkb;
   for (int q = (y - nface) * vb.nt + vb.lt; q < 2 * rows; q += (vb.gy - nface) * vb.nt) {
      const int row = q >> 1;
      const int a = (q & 1) ? d.n[0] - o.i2 : 1 - o.i2;
      if (a < 0 || a >= o.nib) continue;
      const int bb = row % o.njb, c = row / o.njb;
      const int fj = o.j2 + bb, fk = o.k2 + c;
      if (fj == 1 || fj == d.n[1] || (dim == 3 && (fk == 1 || fk == d.n[2]))) continue;
      const long pd = lin32(d, o.i2 + a, fj, fk);
      const double v = interp_point64<TAIL>(o, s, a, bb, c, dim);
      d.f[PGB_F_RES][pd] = v;
      eslot(d, slot)[lin32w(d, o.i2 + a, fj, fk)] = d2f(v);
   }
}

__global__ void k_interp_edges(const pgb_interp_op *ops, const pgb_dbox *boxes, int dim, int slot)
{
   interp_edges_b<false>(hw_blk(), ops, boxes, dim, slot);
}

__device__ double block_sum32(double v, double *sm)
{
   const int t = threadIdx.x + threadIdx.y * blockDim.x;
   const int nt = blockDim.x * blockDim.y;
   for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
   if ((t & 31) == 0) sm[t >> 5] = v;
   __syncthreads();
   if (t < 32) {
      v = (t < (nt >> 5)) ? sm[t] : 0.0;
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
   }
   __syncthreads();
   return v;
}

/* app_MG_residual (num.f:128-175 pattern) in FP64: res = L[u] - rhs at the
 * relaxed points, D = -res and C for the next smoothing block of this
 * level, and call_rr_app's norm (per-box RMS, max over boxes) reduced by the
 * last CTA to finish; with norm_out = 0 (a norm nothing reads) no norm. */
/* call_rr_app over a level (amrd/util.c:39-103): every CTA (split per
 * tile) stores its sum of squared residuals; the CTA that arrives last turns
 * them into per-box RMS values (divided by the box's relaxed-point count) and
 * writes their maximum */
__device__ __forceinline__ void level_rms(const vblk &vb, const pgb_dbox *boxes, const pgb_dlevel &lv,
                                          const pgb_scratch &sc, int split, double acc, double *norm_out,
                                          pgb_trace *trace)
{
   __shared__ double sm[32];
   __shared__ int last;
   acc = block_sum32(acc, sm);
   if (threadIdx.x == 0 && threadIdx.y == 0) sc.partial[vb.x] = acc;
   __threadfence();
   __syncthreads();
   if (threadIdx.x == 0 && threadIdx.y == 0)
      last = (atomicAdd(sc.counter, 1u) == (unsigned)(vb.gx * vb.gy) - 1);
   __syncthreads();
   if (!last) return;
   /* call_rr_app: per-box RMS, max over boxes */
   const int t = threadIdx.x + threadIdx.y * blockDim.x;
   double lres = 0;
   for (int bx = 0; bx < lv.nbox; bx++) {
      double v = 0;
      for (int q = lv.tile_start[bx] * split + t; q < lv.tile_start[bx + 1] * split; q += NT)
         v += __ldcg(&sc.partial[q]);
      v = block_sum32(v, sm);
      if (t == 0) {
         const double r = sqrt(v / boxes[lv.box[bx]].count);
         if (bx == 0) lres = r;
         lres = (r > lres) ? r : lres;
         if (trace) {
            const int n = trace->n;
            if (n < trace->cap) {
               pgb_trace_rec rr = {1, lv.level, bx, 1, r};
               trace->rec[n] = rr;
               trace->n = n + 1;
            } else
               trace->overflow = 1;
         }
      }
   }
   if (t == 0) {
      *norm_out = lres;
      *sc.counter = 0;
   }
}

template <bool PROG, bool TAIL, bool VARS = false>
__device__ __forceinline__ void residual_fast_b(const vblk &vb, const pgb_dbox *boxes, const pgb_dlevel &lv, int pde,
                                                const pgb_scratch &sc, double *norm_out, pgb_trace *trace, int split,
                                                const int *gate)
{
   if (gate && *gate) return;   /* the cycle parity leaves this pass out (no norm is read then) */
   const tile_part tp = tile_split(lv.tiles, lv, split, vb.x);
   const pgb_tile tl = tp.tl;
   const pgb_dbox b = boxes[tl.box];
   const int dim = lv.dim;
   RP(const double) u = b.f[PGB_F_U];
   RP(const double) rhs = b.f[PGB_F_RHS];
   RP(const double) src = b.f[PGB_F_SRC];
   RP(double) res = b.f[PGB_F_RES];
   RP(float) wd = b.w32[W_D];
   RP(float) wc = b.w32[W_C];
   const long sy = b.n[0], sz = (long)b.n[0] * b.n[1];
   double acc = 0;
   const int i = tl.i0 + threadIdx.x, j = tl.j0 + threadIdx.y;
   const int ks = tl.k0 + tp.kk0;
   if (i < b.n[0] && j < b.n[1] && ks < b.n[2]) {
      long p = i + sy * j + sz * ks, q = wq(b, i, j, ks);
      double zm = (dim == 3 && ks > 0) ? u[p - sz] : 0.0, uc = u[p];
#pragma unroll
      for (int kk = 0; kk < PGB_TZ; kk++, p += sz, q += b.wz) {
         const int k = ks + kk;
         if (kk >= tp.nk || k >= b.n[2]) continue;
         const double zp = (dim == 3 && k + 1 < b.n[2]) ? u[p + sz] : 0.0;
         if (interior32(b, i, j, k, dim) && ((b.flags & PGB_BOX_BDY_INTERIOR) || b.cmask_bdy[p])) {
            float c;
            const double lp = lapw(b, u, p, sy, uc, zm, zp, dim);
            const double r = opjac<PROG, VARS>(pde, b, p, lp, uc, src[p], c) - rhs[p];
            res[p] = r;
            wd[q] = d2f(-r);
            if (!VARS || !b.op->jfixed) wc[q] = c;
            if (VARS) coupling_at(b, p, q, lp, uc, src[p]);
            if (norm_out) acc = fma(r, r, acc);
         }
         zm = uc;
         uc = zp;
      }
   }
   if (norm_out) level_rms(vb, boxes, lv, sc, split, acc, norm_out, trace);
}

template <bool PROG, bool VARS = false>
__global__ void __launch_bounds__(NT) k_residual_fast(const pgb_dbox *boxes, pgb_dlevel lv, int pde,
                                                      pgb_scratch sc, double *norm_out,
                                                      pgb_trace *trace, int split, const int *gate)
{
   residual_fast_b<PROG, false, VARS>(hw_blk(), boxes, lv, pde, sc, norm_out, trace, split, gate);
}

/* The convergence norm of a level in a solve with several elliptic
 * variables: each variable's residual pass (k_residual_fast over that
 * variable's view of the boxes) has written its res; this pass sums every
 * variable's squared residual at the relaxed points, the norm of the
 * point-wise hooks of such an application (one sum over all variables per
 * box, amrd/util.c:39-103). */
__global__ void __launch_bounds__(NT) k_norm_vars(const pgb_dbox *boxes, pgb_dlevel lv, pgb_scratch sc,
                                                  double *norm_out, pgb_trace *trace)
{
   const pgb_tile tl = lv.tiles[blockIdx.x];
   const pgb_dbox b = boxes[tl.box];
   const int dim = lv.dim;
   const int i = tl.i0 + threadIdx.x, j = tl.j0 + threadIdx.y;
   const int kz = dim == 3 ? lv.tz : 1;
   double acc = 0;
   if (i < b.n[0] && j < b.n[1])
      for (int kk = 0; kk < kz; kk++) {
         const int k = tl.k0 + kk;
         if (k >= b.n[2]) break;
         const long p = i + (long)b.n[0] * (j + (long)b.n[1] * k);
         if (!relaxed32(b, i, j, k, p, dim)) continue;
         for (int v = 0; v < PGB_NVAR_MAX; v++)
            if (v < lv.nvar) {
               const double r = b.f[PGB_FV(v, PGB_F_RES)][p];
               acc = fma(r, r, acc);
            }
      }
   level_rms(hw_blk(), boxes, lv, sc, 1, acc, norm_out, trace);
}

/* L_op + compute_MG_rhs (amrd/mg.c:271-314) on the cover tiles of the
 * coarsest level, which the coarsest-grid loop smooths by itself */
template <bool PROG, bool VARS = false>
__device__ __forceinline__ void lop_rhs_fast_b(const vblk &vb, const pgb_dbox *boxes, const pgb_dlevel &lv, int pde,
                                               double w0_r)
{
   const pgb_tile tl = lv.ctiles[vb.x];
   const pgb_dbox b = boxes[tl.box];
   const int i = tl.i0 + threadIdx.x, j = tl.j0 + threadIdx.y;
   if (i >= b.n[0] || j >= b.n[1]) return;
   const double *u = b.f[PGB_F_U];
   const long sy = b.n[0], sz = (long)b.n[0] * b.n[1];
   const int kz = lv.dim == 3 ? lv.tz : 1;
#pragma unroll
   for (int kk = 0; kk < PGB_TZ; kk++) {
      const int k = tl.k0 + kk;
      if (kk >= kz || k >= b.n[2]) continue;
      const long p = i + sy * j + sz * k;
      double lopv = 0;
      const int cm = b.cmask_child[p];
      float c;
      if (cm && interior32(b, i, j, k, lv.dim))
         lopv = opjac<PROG, VARS>(pde, b, p, lapm(b, u, p, sy, sz, lv.dim), u[p], b.f[PGB_F_SRC][p], c);
      b.f[PGB_F_RHS][p] = cm ? fma(-b.f[PGB_F_RES][p], w0_r, lopv) : 0.0;
      b.f[PGB_F_LOP][p] = u[p];
   }
}

template <bool PROG, bool VARS = false>
__global__ void __launch_bounds__(NT) k_lop_rhs_fast(const pgb_dbox *boxes, pgb_dlevel lv, int pde,
                                                     double w0_r)
{
   lop_rhs_fast_b<PROG, VARS>(hw_blk(), boxes, lv, pde, w0_r);
}

/* The coarsest-grid loop of the mixed form (amrd/mg.c:172-190: relax the
 * coarsest grids, sync them, until the norm <= crtol x the first norm or
 * MG_max_citer), as defect correction with the whole coarsest level in
 * shared memory of one CTA:
 *   r = L[u] - rhs in FP64 at the relaxed points and its norm (per-box RMS,
 *   max over boxes); stop once it is <= crtol x the first one;
 *   lap E + C E = -r from E = 0 by a fixed number of red-black SOR sweeps in
 *   FP32 (factor omega and the count from the host, enough for a reduction
 *   by crtol), the coarsest boxes' sync applied to E after each sweep;
 *   u += E in FP64, and again from the FP64 residual.
 * FP64 runs at 1/64 of the FP32 rate here, so the FP64 work is one residual
 * pass per correction instead of one per sweep; the FP64 norm decides when
 * to stop, so the result is the FP64 solution to crtol. A correction that
 * fails to halve the FP64 norm means the rounding floor is reached, and the
 * loop stops there. Each thread's points of either colour are listed once
 * (relaxed points only), so no sweep recomputes indices. Sweeps count
 * against MG_max_citer. */
#define CM_MAXB 16
#define CMT 256
template <bool PROG>
__device__ __forceinline__ void coarsest_mixed_b(const pgb_dbox *boxes, const pgb_dlevel &lv, int pde,
                                                 const pgb_copy_op *sync_ops, int nsync, const pgb_coarsest_args &a,
                                                 pgb_trace *trace, int t)
{
   extern __shared__ double dsm[];
   __shared__ double sm[32];
   __shared__ int cb[CM_MAXB], coff[CM_MAXB + 1], ncol[CM_MAXB][2], ncb_s;
   const int dim = lv.dim;
   const bool d3 = dim == 3;
   if (t == 0) {
      int n = 0, o = 0;
      for (int b = 0; b < lv.nbox && n < CM_MAXB; b++) {
         const pgb_dbox &bx = boxes[lv.box[b]];
         if (!(bx.flags & PGB_BOX_COARSEST)) continue;
         cb[n] = b;
         coff[n] = o;
         ncol[n][0] = ncol[n][1] = 0;
         o += bx.n[0] * bx.n[1] * bx.n[2];
         n++;
      }
      coff[n] = o;
      ncb_s = n;
   }
   __syncthreads();
   const int ncb = ncb_s, tot = coff[ncb];
   double *su = dsm;
   float *se = (float *)(dsm + tot), *sd = se + tot, *sc = sd + tot;
   int *sl = (int *)(sc + tot);   /* per box: colour-0 points from the front, colour-1 from the back */
   for (int c = 0; c < ncb; c++) {
      const pgb_dbox &bx = boxes[lv.box[cb[c]]];
      const int n = bx.n[0] * bx.n[1] * bx.n[2];
      for (int q = t; q < n; q += CMT) {
         su[coff[c] + q] = bx.f[PGB_F_U][q];
         se[coff[c] + q] = 0.f;
      }
      const int sy = bx.n[0], sz = bx.n[0] * bx.n[1];
      const int ni = bx.n[0] - 2, nj = bx.n[1] - 2, nk = d3 ? bx.n[2] - 2 : 1;
      for (int q = t; q < ni * nj * nk; q += CMT) {
         const int i = 1 + q % ni, j = 1 + (q / ni) % nj, k = d3 ? 1 + q / (ni * nj) : 0;
         const int p = i + sy * j + sz * k;
         if (!(bx.flags & PGB_BOX_BDY_INTERIOR) && !bx.cmask_bdy[p]) continue;
         /* colour: the pass of num.f:220's red-black order */
         const int col = d3 ? ((i + j + k + 1) & 1) : ((i + j) & 1);
         const int slot = atomicAdd(&ncol[c][col], 1);
         sl[coff[c] + (col ? n - 1 - slot : slot)] = p;
      }
   }
   __syncthreads();
   const float omega = (float)a.omega;
   double ctol = -1.0, res = 0.0, prev = 0.0;
   int sweeps = 0;
   for (;;) {
      /* FP64 residual: D = -r, C, norm */
      double lres = 0;
      for (int c = 0; c < ncb; c++) {
         const pgb_dbox &bx = boxes[lv.box[cb[c]]];
         const double *u = su + coff[c];
         const double *__restrict__ rhs = bx.f[PGB_F_RHS];
         const double *__restrict__ src = bx.f[PGB_F_SRC];
         float *d = sd + coff[c], *cj = sc + coff[c];
         const int *lst = sl + coff[c];
         const int n = bx.n[0] * bx.n[1] * bx.n[2], nrel = ncol[c][0] + ncol[c][1];
         const int sy = bx.n[0], sz = bx.n[0] * bx.n[1];
         double acc = 0;
         for (int q = t; q < nrel; q += CMT) {
            const int p = lst[q < ncol[c][0] ? q : n - nrel + q];
            float cv;
            const double r = opjac<PROG>(pde, bx, p, lapm(bx, u, p, sy, sz, dim), u[p], src[p], cv) - rhs[p];
            d[p] = d2f(-r);
            cj[p] = cv;
            acc = fma(r, r, acc);
         }
         acc = block_sum32(acc, sm);
         if (t == 0) {
            const double r = sqrt(acc / bx.count);
            if (c == 0) lres = r;
            lres = (r > lres) ? r : lres;
            if (trace) {
               const int nt = trace->n;
               if (nt < trace->cap) {
                  pgb_trace_rec *rr = &trace->rec[nt];
                  rr->kind = 0;
                  rr->level = lv.level;
                  rr->box = cb[c];
                  rr->repeat = 1;
                  rr->norm = r;
                  trace->n = nt + 1;
               } else
                  trace->overflow = 1;
            }
         }
      }
      if (t == 0) sm[0] = lres;
      __syncthreads();
      res = sm[0];
      __syncthreads();
      if (ctol < 0)
         ctol = res * a.crtol;
      else if (!(res <= 0.5 * prev))
         break;   /* the last correction did not halve the norm: rounding floor */
      if (res <= ctol || sweeps >= a.max_citer) break;
      prev = res;
      /* FP32 SOR on the correction */
      for (int it = 0; it < a.inner_sweeps && sweeps < a.max_citer; it++, sweeps++) {
         for (int pass = 0; pass < 2; pass++) {
            for (int c = 0; c < ncb; c++) {
               const pgb_dbox &bx = boxes[lv.box[cb[c]]];
               float *e = se + coff[c];
               const float *d = sd + coff[c], *cj = sc + coff[c];
               const int n = bx.n[0] * bx.n[1] * bx.n[2], m = ncol[c][pass];
               const int *lst = sl + coff[c] + (pass ? n - m : 0);
               const int sy = bx.n[0], sz = bx.n[0] * bx.n[1];
               const float ix = bx.fidx2[0], iy = bx.fidx2[1], iz = bx.fidx2[2], j0 = bx.fj0;
               for (int q = t; q < m; q += CMT) {
                  const int p = lst[q];
                  const float ec = e[p], m2 = -2.f * ec, cp = cj[p];
                  float tl = __fmul_rn(__fadd_rn(__fadd_rn(e[p + 1], m2), e[p - 1]), ix);
                  tl = __fmaf_rn(__fadd_rn(__fadd_rn(e[p + sy], m2), e[p - sy]), iy, tl);
                  if (d3) tl = __fmaf_rn(__fadd_rn(__fadd_rn(e[p + sz], m2), e[p - sz]), iz, tl);
                  const float r = __fsub_rn(__fmaf_rn(cp, ec, tl), d[p]);
                  e[p] = __fsub_rn(ec, __fdividef(omega * r, __fadd_rn(j0, cp)));
               }
            }
            __syncthreads();
         }
         for (int o = 0; o < nsync; o++) {   /* PAMR_sync(L,0,MGH,1) over the coarsest grids, on E */
            const pgb_copy_op op = sync_ops[o];
            int cs = -1, cd = -1;
            for (int c = 0; c < ncb; c++) {
               if (lv.box[cb[c]] == op.src_box) cs = c;
               if (lv.box[cb[c]] == op.dst_box) cd = c;
            }
            if (cs < 0 || cd < 0) continue;
            const pgb_dbox &bs = boxes[op.src_box];
            const pgb_dbox &bd = boxes[op.dst_box];
            const int np = op.ni * op.nj * op.nk;
            for (int q = t; q < np; q += CMT) {
               const int aa = q % op.ni, bb = (q / op.ni) % op.nj, cc = q / (op.ni * op.nj);
               se[coff[cd] + lin32(bd, op.i2 + aa, op.j2 + bb, op.k2 + cc)] =
                  se[coff[cs] + lin32(bs, op.i1 + aa, op.j1 + bb, op.k1 + cc)];
            }
            __syncthreads();
         }
      }
      /* u += E where E was set (relaxed and synced points; 0 elsewhere) */
      for (int q = t; q < tot; q += CMT) {
         su[q] += f2d(se[q]);
         se[q] = 0.f;
      }
      __syncthreads();
   }
   for (int c = 0; c < ncb; c++) {
      const pgb_dbox &bx = boxes[lv.box[cb[c]]];
      const int n = bx.n[0] * bx.n[1] * bx.n[2];
      for (int q = t; q < n; q += CMT) bx.f[PGB_F_U][q] = su[coff[c] + q];
   }
   if (t == 0) {
      *a.res_out = res;
      if (a.iters_out) *a.iters_out += sweeps;
   }
}

template <bool PROG>
__global__ void __launch_bounds__(CMT) k_coarsest_mixed(const pgb_dbox *boxes, pgb_dlevel lv, int pde,
                                                        const pgb_copy_op *sync_ops, int nsync,
                                                        pgb_coarsest_args a, pgb_trace *trace)
{
   coarsest_mixed_b<PROG>(boxes, lv, pde, sync_ops, nsync, a, trace, threadIdx.x);
}

/* the cycle parity: 0 -> 1 -> 0 ... at the end of each mixed V-cycle */
__global__ void k_flip(int *parity) { *parity ^= 1; }

extern "C" int pgb_k_flip(int *parity, void *stream)
{
   if (g_tp) return tail_refuse();
   k_flip<<<1, 1, 0, (cudaStream_t)stream>>>(parity);
   return check32("flip");
}

/* one step of the device solve loop (pgb_solve's host loop, amrd/mg.c's
 * solve_elliptics iteration test) */
__global__ void k_solve_step(cudaGraphConditionalHandle h, const double *norm, double *hist, int *it,
                             int min_iter, int max_iter, double tol)
{
   const double r = *norm;
   const int k = *it;
   if (k < max_iter) hist[k] = r;
   *it = k + 1;
   cudaGraphSetConditional(h, ((k + 1 < min_iter || r > tol) && k + 1 < max_iter) ? 1u : 0u);
}

/* ----------------------------------------------------- small-level kernel -- */
/* The passes of the V-cycle over the small levels (pgb_dev.h: pgb_tail_prog)
 * as steps of one launch. One thread-block cluster of up to 16 CTAs of
 * 32 x 8 threads runs them in order: the CTAs share each step's blocks (the
 * blocks of the standalone launch the step replaces, strided over the
 * cluster), the coarsest-grid loop runs in CTA 0 as it does alone, and a
 * cluster barrier (release/acquire at cluster scope) separates a step from
 * the next one that reads what it wrote. Every CTA runs every step and
 * every barrier: the program is a kernel parameter, the same for all, and no
 * thread leaves early. On the small levels each standalone launch costs
 * more than its work; a cluster barrier costs about 0.2 us. */
enum {
   TS_FAS, TS_RELAX, TS_COPYE, TS_DEFECT, TS_UPDATE, TS_UPDDEF, TS_RESID, TS_LOPRHS, TS_CGC, TS_LIN2, TS_IMIX,
   TS_EDGES, TS_RESTRICT, TS_CLEAR, TS_COARSEST
};

__device__ __forceinline__ void cluster_barrier()
{
   asm volatile("barrier.cluster.arrive;\n\tbarrier.cluster.wait;\n" ::: "memory");
}

/* grid mode: every CTA adds one to the counter and waits until it reaches
 * target (the k-th barrier of a launch waits for k x the CTAs); the wait is
 * bounded (about 0.5 s of globaltimer), after which it sets *err and goes on */
__device__ __forceinline__ void grid_barrier(unsigned int *cnt, unsigned int target, int *err)
{
   __syncthreads();
   if (threadIdx.x == 0 && threadIdx.y == 0) {
      __threadfence();
      atomicAdd(cnt, 1u);
      unsigned long long t0 = 0;
      for (int spin = 0;; spin++) {
         unsigned int v;
         asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(cnt) : "memory");
         if (v >= target) break;
         if (spin == 64) t0 = mt_ns();
         if (spin > 64 && mt_ns() - t0 > 500000000ull) {
            atomicExch(err, 4);
            break;
         }
      }
   }
   __syncthreads();
}

/* Mini mode: the arrays of the program's levels staged in shared memory
 * (in = 1: copied in and the shared box table pointed at them; in = 0:
 * grid functions and FP32 arrays copied back). Every thread walks the same
 * regions in the same order (levels, their boxes, fields, FP32 arrays,
 * masks; 16-byte aligned), which is also the order the host sized them in. */
__device__ void tail_stage(const pgb_tail_prog &P, const pgb_dbox *gboxes, pgb_dbox *sbt, unsigned char *m, int in,
                           int lt)
{
   for (int li = 0; li < P.nlev; li++) {
      const pgb_dlevel &g = P.lv[li];
      for (int bi = 0; bi < g.nbox; bi++) {
         const int gb = g.box[bi];
         const pgb_dbox &gx = gboxes[gb];
         const long n = (long)gx.n[0] * gx.n[1] * gx.n[2];
         for (int f = 0; f < PGB_NF; f++) {
            if (!gx.f[f]) continue;
            long long *d = (long long *)m, *a = (long long *)gx.f[f];
            if (in) {
               for (long i = lt; i < n; i += NT) d[i] = a[i];
               if (lt == 0) sbt[gb].f[f] = (double *)d;
            } else
               for (long i = lt; i < n; i += NT) a[i] = d[i];
            m += (n * 8 + 15) / 16 * 16;
         }
         for (int w = 0; w < PGB_NW32; w++) {
            if (!gx.w32[w]) continue;
            const long nw = gx.wz * gx.n[2];
            int *d = (int *)m, *a = (int *)gx.w32[w];
            if (in) {
               for (long i = lt; i < nw; i += NT) d[i] = a[i];
               if (lt == 0) sbt[gb].w32[w] = (float *)d;
            } else
               for (long i = lt; i < nw; i += NT) a[i] = d[i];
            m += (nw * 4 + 15) / 16 * 16;
         }
         for (int c = 0; c < 2; c++) {   /* the masks are only read */
            const uint8_t *a = c ? gx.cmask_bdy : gx.cmask_child;
            if (!a) continue;
            if (in) {
               uint8_t *d = (uint8_t *)m;
               for (long i = lt; i < n; i += NT) d[i] = a[i];
               if (lt == 0) {
                  if (c) sbt[gb].cmask_bdy = d;
                  else sbt[gb].cmask_child = d;
               }
            }
            m += (n + 15) / 16 * 16;
         }
      }
   }
}

template <bool PROG>
__global__ void __launch_bounds__(NT, 1) k_tail(const pgb_dbox *boxes, const __grid_constant__ pgb_tail_prog Pk,
                                                pgb_scratch sc)
{
   const pgb_dbox *const gboxes = boxes;
   const int lt = threadIdx.x + PGB_TX * threadIdx.y;
   const pgb_tail_prog *Pp = &Pk;
   if (Pk.prog_off) {
      /* the program, the box table and the levels' tile and box lists in
       * shared memory: a step's blocks then reach their tile and box without
       * a trip to L2 before their first data load */
      extern __shared__ __align__(16) unsigned char tail_sm[];
      pgb_tail_prog *c = (pgb_tail_prog *)(tail_sm + Pk.prog_off);
      const long long *from = (const long long *)&Pk;
      long long *to = (long long *)c;
      for (int i = lt; i < (int)(sizeof(pgb_tail_prog) / 8); i += NT) to[i] = from[i];
      __syncthreads();   /* before thread 0 points the copy's levels at their lists */
      unsigned char *q = tail_sm + Pk.prog_off + (sizeof(pgb_tail_prog) + 15) / 16 * 16;
      if (Pk.nbox_copy) {
         const int *bf = (const int *)boxes;
         int *bt = (int *)q;
         for (int i = lt; i < (int)(Pk.nbox_copy * sizeof(pgb_dbox) / 4); i += NT) bt[i] = bf[i];
         boxes = (const pgb_dbox *)q;
         q += (Pk.nbox_copy * sizeof(pgb_dbox) + 15) / 16 * 16;
      }
      for (int li = 0; li < Pk.nlev; li++) {
         const pgb_dlevel &g = Pk.lv[li];
         const int *src[4] = {(const int *)g.tiles, (const int *)g.rtiles, (const int *)g.ctiles, g.box};
         const int nw[4] = {g.ntiles * (int)(sizeof(pgb_tile) / 4), g.nrtiles * (int)(sizeof(pgb_tile) / 4),
                            g.nctiles * (int)(sizeof(pgb_tile) / 4), g.nbox};
         for (int a = 0; a < 4; a++) {
            int *d = (int *)q;
            for (int i = lt; i < nw[a]; i += NT) d[i] = src[a][i];
            if (lt == 0) {
               if (a == 0) c->lv[li].tiles = (const pgb_tile *)d;
               else if (a == 1) c->lv[li].rtiles = (const pgb_tile *)d;
               else if (a == 2) c->lv[li].ctiles = (const pgb_tile *)d;
               else c->lv[li].box = d;
            }
            q += ((size_t)nw[a] * 4 + 15) / 16 * 16;
         }
      }
      __syncthreads();
      if (Pk.mini) {   /* the levels' arrays into shared memory, the shared box table pointed at them */
         tail_stage(Pk, gboxes, (pgb_dbox *)boxes, tail_sm + Pk.mini_off, 1, lt);
         __syncthreads();
      }
      Pp = c;
   }
   const pgb_tail_prog &P = *Pp;
   unsigned int nbar = 0;
   for (int s = 0; s < P.nstep; s++) {
      const pgb_tail_step &st = P.step[s];
      const pgb_dlevel &lv = P.lv[st.lev];
      if (st.kind == TS_COARSEST) {
         if (blockIdx.x == 0) coarsest_mixed_b<PROG>(boxes, lv, P.pde, P.csync, P.ncsync, P.ca, 0, lt);
      } else if (!st.solo || blockIdx.x == 0) {
         const int nv = st.gx * st.gy * st.gz, v0 = st.solo ? 0 : blockIdx.x, dv = st.solo ? 1 : gridDim.x;
         for (int v = v0; v < nv; v += dv) {
            vblk vb;
            vb.x = v % st.gx;
            vb.y = (v / st.gx) % st.gy;
            vb.z = v / (st.gx * st.gy);
            vb.gx = st.gx;
            vb.gy = st.gy;
            vb.gz = st.gz;
            vb.lt = lt;
            vb.nt = NT;
            switch (st.kind) {
            case TS_FAS: fas_defect_b<PROG, true>(vb, boxes, lv, P.pde, st.d, st.a[0], st.a[1]); break;
            case TS_RELAX: relax32_b<true>(vb, boxes, lv, st.a[0]); break;
            case TS_COPYE: copy_e_b<true>(vb, boxes, lv, st.a[0]); break;
            case TS_DEFECT: defect32_b<true>(vb, boxes, lv, st.a[0], st.a[1], (const int *)st.ptr, st.a[2]); break;
            case TS_UPDATE: update_b<true>(vb, boxes, lv, st.a[0], st.a[1], st.a[2], st.a[3]); break;
            case TS_UPDDEF:
               update_defect_b<true>(vb, boxes, lv, st.a[0], st.a[1], st.a[2], st.a[3], st.a[4], (const int *)st.ptr,
                                     st.a[5]);
               break;
            case TS_RESID:
               residual_fast_b<PROG, true>(vb, boxes, lv, P.pde, sc, 0, 0, st.a[0], (const int *)st.ptr);
               break;
            case TS_LOPRHS: lop_rhs_fast_b<PROG>(vb, boxes, lv, P.pde, st.d); break;
            case TS_CGC: cgc_mixed_b(vb, boxes, lv, st.d, st.a[0]); break;
            case TS_LIN2: interp_lin2_b<true>(vb, boxes, (const pgb_interp_op *)st.ptr, st.a[0], st.a[1]); break;
            case TS_IMIX: interp_mixed_b<true>(vb, boxes, (const pgb_interp_op *)st.ptr, st.a[0], st.a[1]); break;
            case TS_EDGES: interp_edges_b<true>(vb, (const pgb_interp_op *)st.ptr, boxes, st.a[0], st.a[1]); break;
            case TS_RESTRICT: restrict_b(vb, boxes, (const pgb_restrict_op *)st.ptr, st.a[0], st.a[1]); break;
            case TS_CLEAR: clear_b(vb, boxes, lv, st.a[0]); break;
            default: break;
            }
         }
      }
      if (st.bar == 1) {
         if (P.mini)
            __syncthreads();
         else if (P.grid)
            grid_barrier(P.bar_cnt, ++nbar * gridDim.x, P.err);
         else
            cluster_barrier();
      } else if (st.bar == 2 && blockIdx.x == 0)   /* between two steps of CTA 0 alone */
         __syncthreads();
   }
   if (Pk.mini && Pk.prog_off) {   /* the results back to the device arrays */
      extern __shared__ __align__(16) unsigned char tail_sm[];
      __syncthreads();
      tail_stage(Pk, gboxes, 0, tail_sm + Pk.mini_off, 0, lt);
   }
}


extern "C" void pgb_tail_begin(pgb_tail_prog *p, int pde, int nbox, size_t mini_bytes)
{
   memset(p, 0, sizeof(*p));
   p->pde = pde;
   p->nbox_copy = p->nbox_all = nbox;
   p->mini = mini_bytes > 0;
   p->mini_off = mini_bytes;   /* the staged bytes until the layout is known */
   g_tp = p;
   g_tp_bad = 0;
   g_tp_solo = 0;
}

extern "C" void pgb_tail_set_solo(int on) { g_tp_solo = on != 0; }

extern "C" int pgb_tail_end(void)
{
   pgb_tail_prog *P = g_tp;
   g_tp = 0;
   /* barriers: CTA 0's own between two of its solo steps, the cluster's
    * wherever work changes hands (and after the last step nothing) */
   if (P && !g_tp_bad && (P->mini || !getenv("PGB_TAIL_GLOBALPROG"))) {
      /* shared memory: the coarsest loop's, then the program, the box table
       * (unless it is large) and the levels' tile and box lists */
      size_t q = (P->smem + 15) / 16 * 16 + 16;
      P->prog_off = q;
      q += (sizeof(pgb_tail_prog) + 15) / 16 * 16;
      if (!P->mini && (size_t)P->nbox_copy * sizeof(pgb_dbox) > 48 * 1024) P->nbox_copy = 0;
      q += ((size_t)P->nbox_copy * sizeof(pgb_dbox) + 15) / 16 * 16;
      for (int li = 0; li < P->nlev; li++) {
         const pgb_dlevel &g = P->lv[li];
         q += ((size_t)g.ntiles * sizeof(pgb_tile) + 15) / 16 * 16 + ((size_t)g.nrtiles * sizeof(pgb_tile) + 15) / 16 * 16 +
              ((size_t)g.nctiles * sizeof(pgb_tile) + 15) / 16 * 16 + ((size_t)g.nbox * 4 + 15) / 16 * 16;
      }
      if (P->mini) {   /* then the staged arrays */
         const size_t staged = P->mini_off;
         P->mini_off = q;
         q += staged;
      }
      P->smem_total = q;
      if (q > 200 * 1024) {
         if (P->mini) {
            snprintf(g_err32, sizeof(g_err32), "small-level kernel: %zu bytes of shared memory", q);
            return 1;
         }
         P->prog_off = 0;   /* does not fit: read in place */
      }
   } else if (P)
      P->nbox_copy = 0;
   if (P && !g_tp_bad)
      for (int i = 0; i < P->nstep; i++) {
         pgb_tail_step *t = &P->step[i];
         if (i + 1 == P->nstep)
            t->bar = 0;
         else if (t->bar)
            t->bar = t->solo && P->step[i + 1].solo ? 2 : 1;
      }
   if (g_tp_bad) {
      snprintf(g_err32, sizeof(g_err32), "small-level kernel: %s",
               g_tp_bad == 1 ? "more than PGB_TAIL_MAXSTEP steps or PGB_TAIL_MAXLEV levels"
                             : "a pass it cannot run (FP64 coarsest loop, sync copy or fork)");
      return 1;
   }
   return 0;
}

extern "C" int pgb_tail_recording(void) { return g_tp != 0; }

/* a new step (barrier after it) on level lv (0: none) */
static pgb_tail_step *tadd(int kind, const pgb_dlevel *lv)
{
   pgb_tail_prog *P = g_tp;
   int li = 0;
   if (P->nstep >= PGB_TAIL_MAXSTEP) {
      g_tp_bad = 1;
      return 0;
   }
   if (lv) {
      for (li = 0; li < P->nlev; li++)
         if (P->lv[li].level == lv->level) break;
      if (li == P->nlev) {
         if (P->nlev >= PGB_TAIL_MAXLEV) {
            g_tp_bad = 1;
            return 0;
         }
         P->lv[P->nlev++] = *lv;
      }
   }
   pgb_tail_step *t = &P->step[P->nstep++];
   memset(t, 0, sizeof(*t));
   t->kind = (unsigned char)kind;
   t->lev = (unsigned char)li;
   t->bar = 1;
   t->solo = (unsigned char)(g_tp_solo || kind == TS_COARSEST);
   t->gx = t->gy = t->gz = 1;
   return t;
}


#define TADD(t, kind, lvp)                       \
   pgb_tail_step *t = tadd((kind), (lvp));       \
   if (!t) return 1

extern "C" int pgb_tail_add_restrict(const pgb_plan *p, int field_mask, int res32)
{
   const pgb_restrict_op *h = (const pgb_restrict_op *)p->h_ops, *d = (const pgb_restrict_op *)p->d_ops;
   for (int bt = 0; bt < p->nbatch; bt++) {
      const int n = p->batch_start[bt + 1] - p->batch_start[bt];
      for (int c0 = 0; c0 < n; c0 += 65535) {
         const int m = n - c0 < 65535 ? n - c0 : 65535;
         dim3 g;
         plane_grid(h + p->batch_start[bt] + c0, m, g);
         TADD(t, TS_RESTRICT, 0);
         t->ptr = d + p->batch_start[bt] + c0;
         t->a[0] = field_mask;
         t->a[1] = res32;
         t->gx = (int)g.x;
         t->gy = (int)g.y;
         t->gz = (int)g.z;
      }
   }
   return 0;
}

extern "C" int pgb_tail_add_clear(pgb_dlevel lv, int mask)
{
   TADD(t, TS_CLEAR, &lv);
   t->a[0] = mask;
   t->gx = lv.ntiles;
   return 0;
}

static int tail_attr_set[2];

template <bool PROG>
static cudaError_t tail_attrs()
{
   if (tail_attr_set[PROG]) return cudaSuccess;
   cudaError_t e = cudaFuncSetAttribute(k_tail<PROG>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
   if (e == cudaSuccess) e = cudaFuncSetAttribute(k_tail<PROG>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
   if (e == cudaSuccess) tail_attr_set[PROG] = 1;
   return e;
}

template <bool PROG>
static cudaError_t tail_launch(const pgb_dbox *boxes, const pgb_tail_prog *p, int ncta, pgb_scratch sc,
                               cudaStream_t st)
{
   cudaLaunchConfig_t cfg;
   cudaLaunchAttribute at[1];
   memset(&cfg, 0, sizeof(cfg));
   memset(at, 0, sizeof(at));
   if (p->mini) {
      ncta = 1;
      cfg.numAttrs = 0;
   } else if (p->grid) {
      at[0].id = cudaLaunchAttributeCooperative;
      at[0].val.cooperative = 1;
   } else {
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = (unsigned)ncta;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
   }
   cfg.gridDim = dim3((unsigned)ncta);
   cfg.blockDim = dim3(PGB_TX, PGB_TY);
   cfg.dynamicSmemBytes = p->prog_off ? p->smem_total : p->smem;
   cfg.stream = st;
   cfg.attrs = at;
   cfg.numAttrs = p->mini ? 0 : 1;
   cudaError_t e = tail_attrs<PROG>();
   if (e != cudaSuccess) return e;
   return cudaLaunchKernelEx(&cfg, k_tail<PROG>, boxes, *p, sc);
}

extern "C" int pgb_tail_grid_ctas(void)
{
   int dev = 0, n = 0;
   if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      return 0;
   return n;
}

extern "C" int pgb_k_tail(const pgb_dbox *boxes, const pgb_tail_prog *p, int ncta, pgb_scratch sc, void *stream)
{
   if (!p->nstep) return 0;
   if (p->grid && cudaMemsetAsync(p->bar_cnt, 0, sizeof(unsigned int), (cudaStream_t)stream) != cudaSuccess)
      return check32("tail counter");
   const cudaError_t e = p->pde == PGB_OPK_PROGRAM ? tail_launch<true>(boxes, p, ncta, sc, (cudaStream_t)stream)
                                                   : tail_launch<false>(boxes, p, ncta, sc, (cudaStream_t)stream);
   if (e != cudaSuccess) {
      snprintf(g_err32, sizeof(g_err32), "small-level kernel: %s", cudaGetErrorString(e));
      return 1;
   }
   return check32("tail");
}

extern "C" int pgb_tail_max_cluster(size_t smem)
{
   if (tail_attrs<false>() != cudaSuccess || tail_attrs<true>() != cudaSuccess) return 0;
   for (int cs = 16; cs >= 1; cs /= 2) {
      cudaLaunchConfig_t cfg;
      cudaLaunchAttribute at[1];
      memset(&cfg, 0, sizeof(cfg));
      memset(at, 0, sizeof(at));
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = (unsigned)cs;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.gridDim = dim3((unsigned)cs);
      cfg.blockDim = dim3(PGB_TX, PGB_TY);
      cfg.dynamicSmemBytes = smem;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      int n0 = 0, n1 = 0;
      if (cudaOccupancyMaxActiveClusters(&n0, k_tail<false>, &cfg) == cudaSuccess &&
          cudaOccupancyMaxActiveClusters(&n1, k_tail<true>, &cfg) == cudaSuccess && n0 >= 1 && n1 >= 1)
         return cs;
      cudaGetLastError();
   }
   return 0;
}

/* ------------------------------------------------------------ launchers -- */
extern "C" int pgb_k_fas_defect(const pgb_dbox *boxes, pgb_dlevel lv, int pde, double w0_r, int cover,
                                void *stream)
{
   const int n = cover ? lv.nctiles : lv.ntiles;
   if (!n) return 0;
   const int sp = split_for(lv, n);
   if (g_tp) {
      TADD(t, TS_FAS, &lv);
      t->a[0] = cover;
      t->a[1] = sp;
      t->d = w0_r;
      t->gx = n * sp;
      return 0;
   }
   if (lv.nvar > 1)   /* one variable of several (a program operator) */
      k_fas_defect<true, true><<<n * sp, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream>>>(boxes, lv, pde, w0_r, cover,
                                                                                        sp);
   else
      OPLAUNCH(k_fas_defect, pde, n * sp, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream, boxes, lv, pde, w0_r, cover,
               sp);
   return check32("fas_defect");
}

extern "C" int pgb_k_defect32(const pgb_dbox *boxes, pgb_dlevel lv, int slot, const int *gate, int gval,
                              void *stream)
{
   if (!lv.ntiles) return 0;
   const int sp = split_for(lv, lv.ntiles);
   if (g_tp) {
      TADD(t, TS_DEFECT, &lv);
      t->a[0] = slot;
      t->a[1] = sp;
      t->a[2] = gval;
      t->ptr = gate;
      t->gx = lv.ntiles * sp;
      return 0;
   }
   k_defect32<<<lv.ntiles * sp, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream>>>(boxes, lv, slot, sp, gate,
                                                                                 gval);
   return check32("defect32");
}

/* nsweep FP32 sweeps of level L: fuse = 0 two global-memory colour passes
 * per sweep (in place, slot W_E); 1 or 2 = sweeps per launch of the
 * shared-memory kernel, 3 = the one-pass marching kernel (3-D), 4 or 5 =
 * the TMA-staged sweep, 6 or 7 = two TMA-staged sweeps per launch (an odd
 * last sweep runs alone in the shared-memory kernel). The fused
 * kernels read one slot and write the other; *slot says where the
 * correction starts and, on return, where it ends, which the block's
 * consumers (sync, defect, update) read. */
extern "C" int pgb_k_sweep32(const pgb_dbox *boxes, pgb_dlevel lv, int nsweep, int fuse, int *slot,
                             void *stream)
{
   int done = 0, src = *slot, dst = src == W_E ? W_E2 : W_E;
   if (!lv.ntiles) return 0;
   if (g_tp) {   /* the small-level kernel relaxes by colour passes in place */
      if (fuse > 0) return tail_refuse();
      if (src != W_E) {
         TADD(t, TS_COPYE, &lv);
         t->a[0] = src;
         t->gx = lv.ntiles;
         *slot = W_E;
      }
      for (; done < nsweep; done++)
         for (int pass = 0; pass < 2; pass++) {
            TADD(t, TS_RELAX, &lv);
            t->a[0] = pass;
            t->gx = lv.nrtiles;
         }
      return 0;
   }
   if (fuse <= 0) {   /* in place, one launch per colour pass */
      if (src != W_E) {
         k_copy_e<<<lv.ntiles, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream>>>(boxes, lv, src);
         if (check32("copy_e")) return 1;
         *slot = W_E;
      }
      for (; done < nsweep; done++) {
         k_relax32<<<lv.nrtiles, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream>>>(boxes, lv, 0);
         if (check32("relax32")) return 1;
         k_relax32<<<lv.nrtiles, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream>>>(boxes, lv, 1);
         if (check32("relax32")) return 1;
      }
      return 0;
   }
   /* fused launches alternate between the two correction slots */
   while (done < nsweep) {
      if ((fuse == 4 || fuse == 5 || ((fuse == 6 || fuse == 7) && nsweep - done >= 2)) && lv.dim == 3 && lv.tmaps &&
          lv.nmtiles) {
         if (sweep32t(boxes, lv, lv.tmaps, src, dst, lv.err, (cudaStream_t)stream)) return 1;
         done += fuse >= 6 ? 2 : 1;
         const int t = src;
         src = dst;
         dst = t;
         continue;
      }
      if (fuse == 3 && lv.dim == 3) {
         k_sweep32z<<<lv.nztiles, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream>>>(boxes, lv, src, dst);
         done += 1;
      } else if (fuse >= 2 && fuse != 3 && nsweep - done >= 2) {
         k_sweep32<2><<<lv.ntiles, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream>>>(boxes, lv, src, dst);
         done += 2;
      } else {
         k_sweep32<1><<<lv.ntiles, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream>>>(boxes, lv, src, dst);
         done += 1;
      }
      if (check32("sweep32")) return 1;
      const int t = src;
      src = dst;
      dst = t;
   }
   *slot = src;
   return 0;
}

extern "C" int pgb_k_solve_step(unsigned long long handle, const double *norm, double *hist, int *it,
                                int min_iter, int max_iter, double tol, void *stream)
{
   k_solve_step<<<1, 1, 0, (cudaStream_t)stream>>>((cudaGraphConditionalHandle)handle, norm, hist, it,
                                                   min_iter, max_iter, tol);
   return check32("solve_step");
}

extern "C" int pgb_k_update(const pgb_dbox *boxes, pgb_dlevel lv, int post, int slot, int zslot,
                            void *stream)
{
   if (!lv.ntiles) return 0;
   const int sp = split_for(lv, lv.ntiles);
   if (g_tp) {
      TADD(t, TS_UPDATE, &lv);
      t->a[0] = post;
      t->a[1] = slot;
      t->a[2] = zslot;
      t->a[3] = sp;
      t->gx = lv.ntiles * sp;
      return 0;
   }
   k_update<<<lv.ntiles * sp, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream>>>(boxes, lv, post, slot, zslot,
                                                                               sp);
   return check32("update");
}

extern "C" int pgb_k_update_defect(const pgb_dbox *boxes, pgb_dlevel lv, int post, int slot, int zslot,
                                   int defect, const int *gate, int gval, void *stream)
{
   if (!lv.ntiles) return 0;
   if (zslot == slot) {
      snprintf(g_err32, sizeof(g_err32), "update_defect: the zeroed slot is the one read");
      return 1;
   }
   const int sp = split_for(lv, lv.ntiles);
   if (g_tp) {
      TADD(t, TS_UPDDEF, &lv);
      t->a[0] = post;
      t->a[1] = slot;
      t->a[2] = zslot;
      t->a[3] = sp;
      t->a[4] = defect;
      t->a[5] = gval;
      t->ptr = gate;
      t->gx = lv.ntiles * sp;
      return 0;
   }
   k_update_defect<<<lv.ntiles * sp, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream>>>(boxes, lv, post, slot, zslot,
                                                                                      sp, defect, gate, gval);
   return check32("update_defect");
}

extern "C" int pgb_k_zero32(const pgb_dbox *boxes, pgb_dlevel lv, void *stream)
{
   if (g_tp) return tail_refuse();
   if (!lv.ntiles) return 0;
   k_zero32<<<lv.ntiles, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream>>>(boxes, lv);
   return check32("zero32");
}

extern "C" int pgb_k_copy32(const pgb_dbox *boxes, const pgb_plan *p, int slot, void *stream)
{
   if (g_tp) return tail_refuse();
   const pgb_copy_op *h = (const pgb_copy_op *)p->h_ops, *d = (const pgb_copy_op *)p->d_ops;
   for (int bt = 0; bt < p->nbatch; bt++) {
      const int n = p->batch_start[bt + 1] - p->batch_start[bt];
      for (int c0 = 0; c0 < n; c0 += 65535) {
         const int m = n - c0 < 65535 ? n - c0 : 65535;
         dim3 g;
         plane_grid(h + p->batch_start[bt] + c0, m, g);
         k_copy32<<<g, 256, 0, (cudaStream_t)stream>>>(boxes, d + p->batch_start[bt] + c0, slot);
         if (check32("copy32")) return 1;
      }
   }
   return 0;
}

extern "C" int pgb_k_cgc_mixed(const pgb_dbox *boxes, pgb_dlevel lv, double inv_w0, void *stream)
{
   if (!lv.nctiles) return 0;
   const int sp = split_for(lv, lv.nctiles);
   if (g_tp) {
      TADD(t, TS_CGC, &lv);
      t->a[0] = sp;
      t->d = inv_w0;
      t->gx = lv.nctiles * sp;
      return 0;
   }
   k_cgc_mixed<<<lv.nctiles * sp, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream>>>(boxes, lv, inv_w0, sp);
   return check32("cgc_mixed");
}

/* With one batch (ops with disjoint destinations) and a side stream, the
 * FP64 edge kernel runs beside the FP32 kernel: they write disjoint points
 * (the FP32 kernel leaves the face rows and x-ends of all-relaxed boxes to
 * it) and only read the coarse level. fork/join are events without timing. */
extern "C" int pgb_k_interp_mixed(const pgb_dbox *boxes, const pgb_plan *p, int dim, int slot, void *stream,
                                  void *side, void *fork, void *join)
{
   const pgb_interp_op *h = (const pgb_interp_op *)p->h_ops, *d = (const pgb_interp_op *)p->d_ops;
   if (g_tp) {   /* no fork: the two kernels of a batch as steps with no barrier between them */
      for (int bt = 0; bt < p->nbatch; bt++) {
         const int n = p->batch_start[bt + 1] - p->batch_start[bt];
         for (int c0 = 0; c0 < n; c0 += 65535) {
            const int m = n - c0 < 65535 ? n - c0 : 65535;
            const pgb_interp_op *hb = h + p->batch_start[bt] + c0;
            dim3 g;
            long mr = 1, mf = 1;
            int lin2 = 1, mi = 1;
            row_grid(hb, m, g);
            for (int i = 0; i < m; i++) {
               if ((long)hb[i].njb * hb[i].nkb > mr) mr = (long)hb[i].njb * hb[i].nkb;
               if (hb[i].irho != 2 || (hb[i].ord != 2 && (hb[i].nii >= 4 || hb[i].nji >= 4 || (dim == 3 && hb[i].nki >= 4))))
                  lin2 = 0;
               if (hb[i].nib > mi) mi = hb[i].nib;
               if (2L * (hb[i].njb + hb[i].nkb) > mf) mf = 2L * (hb[i].njb + hb[i].nkb);
            }
            TADD(t, lin2 ? TS_LIN2 : TS_IMIX, 0);
            t->ptr = d + p->batch_start[bt] + c0;
            t->a[0] = dim;
            t->a[1] = slot;
            t->gx = (int)g.x;
            t->gy = (int)g.y;
            t->gz = (int)g.z;
            t->bar = 0;   /* the edge step writes other points and reads only the coarse level */
            long gy = mf + (2 * mr + 127) / 128;
            TADD(t2, TS_EDGES, 0);
            t2->ptr = d + p->batch_start[bt] + c0;
            t2->a[0] = dim;
            t2->a[1] = slot;
            t2->gx = (mi + 127) / 128;
            t2->gy = (int)(gy > 65535 ? 65535 : gy);
            t2->gz = m;
         }
      }
      return 0;
   }
   const bool par = side && p->nbatch == 1;
   cudaStream_t es = par ? (cudaStream_t)side : (cudaStream_t)stream;
   if (par) {
      if (cudaEventRecord((cudaEvent_t)fork, (cudaStream_t)stream) != cudaSuccess ||
          cudaStreamWaitEvent(es, (cudaEvent_t)fork, 0) != cudaSuccess)
         return check32("interp_mixed fork");
   }
   for (int bt = 0; bt < p->nbatch; bt++) {
      const int n = p->batch_start[bt + 1] - p->batch_start[bt];
      for (int c0 = 0; c0 < n; c0 += 65535) {
         const int m = n - c0 < 65535 ? n - c0 : 65535;
         const pgb_interp_op *hb = h + p->batch_start[bt] + c0;
         dim3 g;
         long mr = 1;
         int lin2 = 1;
         row_grid(hb, m, g);
         for (int i = 0; i < m; i++) {
            if ((long)hb[i].njb * hb[i].nkb > mr) mr = (long)hb[i].njb * hb[i].nkb;
            if (hb[i].irho != 2 || (hb[i].ord != 2 && (hb[i].nii >= 4 || hb[i].nji >= 4 || (dim == 3 && hb[i].nki >= 4))))
               lin2 = 0;
         }
         if (lin2)
            k_interp_lin2<<<g, 128, 0, (cudaStream_t)stream>>>(boxes, d + p->batch_start[bt] + c0, dim, slot);
         else
            k_interp_mixed<<<g, 128, 0, (cudaStream_t)stream>>>(boxes, d + p->batch_start[bt] + c0, dim, slot);
         if (check32("interp_mixed")) return 1;
         {
            int mi = 1;
            long mf = 1;
            for (int i = 0; i < m; i++) {
               if (hb[i].nib > mi) mi = hb[i].nib;
               if (2L * (hb[i].njb + hb[i].nkb) > mf) mf = 2L * (hb[i].njb + hb[i].nkb);
            }
            long gy = mf + (2 * mr + 127) / 128;   /* face rows, then x-end chunks */
            k_interp_edges<<<dim3((unsigned)((mi + 127) / 128), (unsigned)(gy > 65535 ? 65535 : gy), (unsigned)m),
                             128, 0, es>>>(d + p->batch_start[bt] + c0, boxes, dim, slot);
            if (check32("interp_edges")) return 1;
         }
      }
   }
   if (par) {
      if (cudaEventRecord((cudaEvent_t)join, es) != cudaSuccess ||
          cudaStreamWaitEvent((cudaStream_t)stream, (cudaEvent_t)join, 0) != cudaSuccess)
         return check32("interp_mixed join");
   }
   return 0;
}

extern "C" int pgb_k_residual_fast(const pgb_dbox *boxes, pgb_dlevel lv, int pde, pgb_scratch sc,
                                   double *norm_out, pgb_trace *trace, const int *gate, void *stream)
{
   if (!lv.ntiles) return 0;
   int sp = split_for(lv, lv.ntiles);
   while (sp > 1 && (long)lv.ntiles * sp > sc.npartial) sp /= 2;   /* one partial sum per CTA */
   if (g_tp) {   /* a residual whose norm nothing reads */
      if (norm_out || trace) return tail_refuse();
      TADD(t, TS_RESID, &lv);
      t->a[0] = sp;
      t->ptr = gate;
      t->gx = lv.ntiles * sp;
      return 0;
   }
   if (lv.nvar > 1)   /* one variable of several (a program operator) */
      k_residual_fast<true, true><<<lv.ntiles * sp, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream>>>(
         boxes, lv, pde, sc, norm_out, trace, sp, gate);
   else
      OPLAUNCH(k_residual_fast, pde, lv.ntiles * sp, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream, boxes, lv, pde, sc,
               norm_out, trace, sp, gate);
   return check32("residual_fast");
}

extern "C" int pgb_k_relax32_vars(pgb_vtabs vt, pgb_dlevel lv, int pass, void *stream)
{
   if (!lv.nrtiles) return 0;
   if (g_tp) return tail_refuse();
   k_relax32_vars<<<lv.nrtiles, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream>>>(vt, lv, pass);
   return check32("relax32_vars");
}

extern "C" int pgb_k_couplings(const pgb_dbox *boxes, pgb_dlevel lv, void *stream)
{
   if (!lv.ntiles) return 0;
   if (g_tp) return tail_refuse();
   k_couplings<<<lv.ntiles, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream>>>(boxes, lv);
   return check32("couplings");
}

extern "C" int pgb_k_norm_vars(const pgb_dbox *boxes, pgb_dlevel lv, pgb_scratch sc, double *norm_out,
                               pgb_trace *trace, void *stream)
{
   if (!lv.ntiles) return 0;
   if (g_tp) return tail_refuse();
   k_norm_vars<<<lv.ntiles, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream>>>(boxes, lv, sc, norm_out, trace);
   return check32("norm_vars");
}

extern "C" int pgb_k_lop_rhs_fast(const pgb_dbox *boxes, pgb_dlevel lv, int pde, double w0_r,
                                  void *stream)
{
   if (!lv.nctiles) return 0;
   if (g_tp) {
      TADD(t, TS_LOPRHS, &lv);
      t->d = w0_r;
      t->gx = lv.nctiles;
      return 0;
   }
   if (lv.nvar > 1)   /* one variable of several (a program operator) */
      k_lop_rhs_fast<true, true><<<lv.nctiles, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream>>>(boxes, lv, pde, w0_r);
   else
      OPLAUNCH(k_lop_rhs_fast, pde, lv.nctiles, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream, boxes, lv, pde, w0_r);
   return check32("lop_rhs_fast");
}

/* returns 1 (nothing launched) when the coarsest level does not fit on chip */
extern "C" int pgb_k_coarsest_mixed(const pgb_dbox *boxes, pgb_dlevel lv, int pde, const pgb_plan *sync,
                                    pgb_coarsest_args a, pgb_trace *trace, void *stream)
{
   /* u (FP64), E, D, C (FP32) and the point lists (int) per point */
   const size_t smem = (size_t)a.smem_points * (sizeof(double) + 3 * sizeof(float) + sizeof(int));
   static int attr_set = 0;
   if (a.smem_points <= 0 || a.ncoarse > CM_MAXB || smem > 200 * 1024) return 1;
   if (g_tp) {   /* one coarsest loop per program, run by CTA 0 */
      if (trace || g_tp->ca.res_out) return tail_refuse() ? -1 : -1;
      TADD(t, TS_COARSEST, &lv);
      (void)t;
      g_tp->ca = a;
      g_tp->csync = (const pgb_copy_op *)sync->d_ops;
      g_tp->ncsync = sync->nops;
      if (smem > g_tp->smem) g_tp->smem = smem;
      return 0;
   }
   if (!attr_set) {
      cudaFuncSetAttribute(k_coarsest_mixed<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
      cudaFuncSetAttribute(k_coarsest_mixed<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
      attr_set = 1;
   }
   OPLAUNCH(k_coarsest_mixed, pde, 1, CMT, smem, (cudaStream_t)stream, boxes, lv, pde,
            (const pgb_copy_op *)sync->d_ops, sync->nops, a, trace);
   return check32("coarsest_mixed") ? -1 : 0;
}
