/*
 * FP64 multigrid kernels of libpamr_gb300 (sm_103a).
 *
 * This translation unit is compiled with -fmad=false: every product and sum
 * is rounded separately, in the order of the reference's Fortran/C
 * expressions, so results match the reference's CPU arithmetic bit for bit
 * (examples/nbs/num.f:85-246 pattern for the operators, src/m_util_r8.f for
 * the transfer operators, amrd/mg.c:242-355 for the FAS bookkeeping).
 * Only the norm reductions are summed in a different (fixed, deterministic)
 * order, so norms agree to about 1e-15 relative.
 *
 * Layout: every grid function of every box is a dense float64 array with x
 * fastest (Fortran u(Nx,Ny,Nz)); a level's boxes are covered by a list of
 * tiles, one CTA per tile. All boxes of a level are processed by one launch.
 */
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "pgb_dev.h"
#include "pgb_opgrid.cuh"
#include "pgb_op.cuh"
#include "pgb_weights.cuh"

namespace cg = cooperative_groups;

static __thread char g_err[256];
static unsigned long long g_launches = 0;

extern "C" const char *pgb_dev_error(void) { return g_err; }
extern "C" unsigned long long pgb_dev_launches(void) { return g_launches; }

#define LAUNCHED(n) (g_launches += (unsigned long long)(n))

/* while the small-level kernel records (pgb_dev.h): an FP64 pass it runs is
 * recorded (rc = 0 or 1 returned), one it cannot run refuses */
static int tail_note(int rc, const char *what)
{
   if (rc) snprintf(g_err, sizeof(g_err), "%s: %s", what, pgb_dev_error32());
   return rc;
}
#define TAIL_REFUSE(what)                                                                 do {                                                                                       if (pgb_tail_recording()) {                                                                snprintf(g_err, sizeof(g_err), "%s: not a pass of the small-level kernel", what);          return 1;                                                                            }                                                                                    } while (0)

static int check(const char *what)
{
   cudaError_t e = cudaGetLastError();
   if (e != cudaSuccess) {
      snprintf(g_err, sizeof(g_err), "%s: %s", what, cudaGetErrorString(e));
      return 1;
   }
   return 0;
}

extern "C" int pgb_dev_sync(void *stream)
{
   cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
   if (e != cudaSuccess) {
      snprintf(g_err, sizeof(g_err), "stream sync: %s", cudaGetErrorString(e));
      return 1;
   }
   return 0;
}

#define NT (PGB_TX * PGB_TY)

/* launches the instantiation of an operator kernel for the level
 * operator's form: compiled built-in (PROG = false) or program (true) */
#define OPLAUNCH(kern, pde, grid, blk, smem, st, ...)                                   \
   do {                                                                                 \
      if ((pde) == PGB_OPK_PROGRAM) kern<true><<<(grid), (blk), (smem), (st)>>>(__VA_ARGS__); \
      else kern<false><<<(grid), (blk), (smem), (st)>>>(__VA_ARGS__);                   \
   } while (0)

/* ------------------------------------------------------------ operators -- */
/* 2*pi and 5*2*pi, the constants of the conformal-factor hook */
#define TWO_PI 6.283185307179586
#define TEN_PI 31.41592653589793

/* one term of num.f:113-115: num/dx^2 (a product when 1/dx^2 is exact) */
__device__ __forceinline__ double dterm(const pgb_dbox &b, double num, int d)
{
   return (b.flags & PGB_BOX_POW2DX) ? num * b.idx2[d] : div_known(num, b.dx2[d], b.idx2[d]);
}

/* lap(u) at linear index p, num.f:113-115 order */
__device__ __forceinline__ double lap64(const pgb_dbox &b, const double *u, long p, int dim)
{
   long sy = b.n[0], sz = (long)b.n[0] * b.n[1];
   double c = u[p];
   double t = dterm(b, u[p + 1] - 2 * c + u[p - 1], 0) + dterm(b, u[p + sy] - 2 * c + u[p - sy], 1);
   if (dim == 3) t = t + dterm(b, u[p + sz] - 2 * c + u[p - sz], 2);
   return t;
}

/* L[u] at point p of box b from t = lap u: the built-in operators in the
 * order of their hooks, or the box's operator program (pgb_op.cuh) */
template <bool PROG>
__device__ __forceinline__ double op64(int pde, const pgb_dbox &b, long p, double t, double u, double s)
{
   if (PROG) return pgb_prog_L(b, t, u, s, p);
   if (pde == PGB_OPK_CONFORMAL) {
      double p2 = u * u, p4 = p2 * p2;
      return t + TWO_PI * s * (p4 * u);
   }
   if (pde == PGB_OPK_LAPSE) return t - s * u;
   return t - s;
}

/* dL/du at point p (the relaxation's Newton diagonal) */
template <bool PROG>
__device__ __forceinline__ double jac64(int pde, const pgb_dbox &b, long p, double u, double s)
{
   if (PROG) return pgb_prog_J(b, u, s, p);
   if (pde == PGB_OPK_CONFORMAL) {
      double p2 = u * u;
      return b.j0 + TEN_PI * s * (p2 * p2);
   }
   if (pde == PGB_OPK_LAPSE) return b.j0 - s;
   return b.j0;
}

__device__ __forceinline__ bool interior(const pgb_dbox &b, int i, int j, int k, int dim)
{
   return i >= 1 && i <= b.n[0] - 2 && j >= 1 && j <= b.n[1] - 2 &&
          (dim == 2 ? k == 0 : (k >= 1 && k <= b.n[2] - 2));
}

/* deterministic block sum of one double per thread (fixed tree) */
__device__ double block_sum(double v, double *sm)
{
   int t = threadIdx.x + threadIdx.y * blockDim.x;
   int nt = blockDim.x * blockDim.y;
   for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
   if ((t & 31) == 0) sm[t >> 5] = v;
   __syncthreads();
   if (t < 32) {
      v = (t < (nt >> 5)) ? sm[t] : 0.0;
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
   }
   __syncthreads();
   return v;   /* valid in thread 0 */
}

/* call_rr_app (amrd/util.c:73-103): per-box RMS, max over the level's boxes.
 * Runs in the last CTA of a launch; sums the per-tile partials in a fixed
 * order. npart = 1 (residual) or 2 (relax: two colour passes). */
__device__ void finalize_norm(const pgb_dbox *boxes, const pgb_dlevel &lv, const int *tstart,
                              int ntiles, int npart, pgb_scratch sc, double *norm_out,
                              pgb_trace *trace, int kind, double *sm)
{
   int t = threadIdx.x + threadIdx.y * blockDim.x;
   int nt = blockDim.x * blockDim.y;
   double lres = 0;
   for (int b = 0; b < lv.nbox; b++) {
      double v = 0;
      for (int q = 0; q < npart; q++)
         for (int s = tstart[b] + t; s < tstart[b + 1]; s += nt) v += __ldcg(&sc.partial[q * ntiles + s]);
      v = block_sum(v, sm);
      if (t == 0) {
         const pgb_dbox &bx = boxes[lv.box[b]];
         double r = sqrt(v / bx.count);
         if (b == 0) lres = r;
         lres = (r > lres) ? r : lres;
         if (trace) {
            int n = trace->n;
            if (n < trace->cap) {
               pgb_trace_rec rr = {kind, lv.level, b, 1, r};
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

/* true in exactly one CTA: the last one to finish */
__device__ bool last_block(pgb_scratch sc, int *flag)
{
   __threadfence();
   __syncthreads();
   if (threadIdx.x == 0 && threadIdx.y == 0) {
      unsigned int total = gridDim.x * gridDim.y;
      unsigned int v = atomicAdd(sc.counter, 1u);
      *flag = (v == total - 1);
   }
   __syncthreads();
   return *flag != 0;
}

/* ------------------------------------------------ several variables -- */
/* The hooks of an application with several elliptic variables update them
 * point by point (AMRD calls one relax per grid for all of them, amrd/mg.c:
 * 135-141): at each point of the colour, variable 0, 1, ... in turn, each
 * from the others' current values at the point; the norm sums every
 * variable's squared residual. Program operators only (one per variable,
 * b.op[v]). */
__device__ __forceinline__ void load_vars(const pgb_dbox &b, int nvar, long p, double *uv)
{
   for (int v = 0; v < nvar; v++) uv[v] = b.f[PGB_FV(v, PGB_F_U)][p];
}

/* Gauss-Seidel at point p over the variables; returns the sum of the
 * squared in-sweep residuals */
__device__ double relax_vars(const pgb_dbox &b, int nvar, long p, int dim)
{
   double uv[PGB_NVAR_MAX], acc = 0;
   const pgb_srcv sv = pgb_load_src(b.op->nsrc, b, p, b.f[PGB_F_SRC][p]);
   load_vars(b, nvar, p, uv);
   for (int v = 0; v < nvar; v++) {
      double *u = b.f[PGB_FV(v, PGB_F_U)];
      const double r = pgb_prog_Lv(b, v, lap64(b, u, p, dim), uv, sv) - b.f[PGB_FV(v, PGB_F_RHS)][p];
      const double jac = pgb_prog_Jv(b, v, uv, sv);
      uv[v] = uv[v] - r / jac;
      u[p] = uv[v];
      acc += r * r;
   }
   return acc;
}

/* The mixed form's coarsest-grid loop with several variables: Newton at
 * point p on all variables together (the point's nvar x nvar Jacobian: each
 * program's diagonal and, by differentiating it, its coupling to the other
 * variables; Gaussian elimination with partial pivoting), over-relaxed by
 * om. Where the coupling dominates the diagonal (coarse grids of a large
 * domain) the point-wise sweeps over one variable after the other reduce
 * the modes it couples by little per sweep; this takes them in one.
 * Returns the sum of the squared residuals before the update. */
__device__ double relax_vars_block(const pgb_dbox &b, int nvar, long p, int dim, double om)
{
   double uv[PGB_NVAR_MAX], r[PGB_NVAR_MAX], J[PGB_NVAR_MAX][PGB_NVAR_MAX], acc = 0;
   const pgb_srcv sv = pgb_load_src(b.op->nsrc, b, p, b.f[PGB_F_SRC][p]);
   load_vars(b, nvar, p, uv);
   for (int v = 0; v < nvar; v++) {
      const pgb_dop *o = b.op + v;
      const double lp = lap64(b, b.f[PGB_FV(v, PGB_F_U)], p, dim);
      r[v] = pgb_prog_Lv(b, v, lp, uv, sv) - b.f[PGB_FV(v, PGB_F_RHS)][p];
      acc += r[v] * r[v];
      for (int k = 0; k < nvar; k++)
         J[v][k] = k == v ? pgb_prog_Jv(b, v, uv, sv) : pgb_prog_dvar(o->lcode, o->cst, lp, b.j0, uv[v], uv, sv, k);
   }
   for (int c = 0; c < nvar; c++) {
      int piv = c;
      for (int i = c + 1; i < nvar; i++)
         if (fabs(J[i][c]) > fabs(J[piv][c])) piv = i;
      if (piv != c) {
         for (int k = 0; k < nvar; k++) {
            const double x = J[c][k];
            J[c][k] = J[piv][k];
            J[piv][k] = x;
         }
         const double x = r[c];
         r[c] = r[piv];
         r[piv] = x;
      }
      for (int i = c + 1; i < nvar; i++) {
         const double f = J[i][c] / J[c][c];
         for (int k = c; k < nvar; k++) J[i][k] -= f * J[c][k];
         r[i] -= f * r[c];
      }
   }
   for (int c = nvar - 1; c >= 0; c--) {
      double x = r[c];
      for (int k = c + 1; k < nvar; k++) x -= J[c][k] * r[k];
      r[c] = x / J[c][c];
   }
   for (int v = 0; v < nvar; v++) b.f[PGB_FV(v, PGB_F_U)][p] = uv[v] - om * r[v];
   return acc;
}

/* residual of every variable at point p (res_v = L_v - rhs_v); returns the
 * sum of their squares */
__device__ double residual_vars(const pgb_dbox &b, int nvar, long p, int dim)
{
   double uv[PGB_NVAR_MAX], acc = 0;
   const pgb_srcv sv = pgb_load_src(b.op->nsrc, b, p, b.f[PGB_F_SRC][p]);
   load_vars(b, nvar, p, uv);
   for (int v = 0; v < nvar; v++) {
      const double r = pgb_prog_Lv(b, v, lap64(b, b.f[PGB_FV(v, PGB_F_U)], p, dim), uv, sv) -
                       b.f[PGB_FV(v, PGB_F_RHS)][p];
      b.f[PGB_FV(v, PGB_F_RES)][p] = r;
      acc += r * r;
   }
   return acc;
}

/* ---------------------------------------------------------------- relax -- */
/* one colour pass of relax (num.f:216-241); pass 1 finalizes the norm */
template <bool PROG>
__global__ void __launch_bounds__(NT) k_relax(const pgb_dbox *boxes, pgb_dlevel lv, int pde,
                                              int pass, pgb_scratch sc, double *norm_out,
                                              pgb_trace *trace)
{
   __shared__ double sm[32];
   __shared__ int flag;
   const pgb_tile tl = lv.rtiles[blockIdx.x];
   const pgb_dbox b = boxes[tl.box];
   const int dim = lv.dim;
   double *u = b.f[PGB_F_U];
   const double *rhs = b.f[PGB_F_RHS], *src = b.f[PGB_F_SRC];
   double acc = 0;
   int j = tl.j0 + threadIdx.y;
   int kz = dim == 3 ? lv.rtz : 1;
   for (int kk = 0; kk < kz; kk++) {
      int k = tl.k0 + kk;
      int par = dim == 3 ? ((j + k + 1 + pass) & 1) : ((j + pass) & 1);
      int i = tl.i0 + 2 * threadIdx.x + par;
      if (!interior(b, i, j, k, dim)) continue;
      long p = i + (long)b.n[0] * (j + (long)b.n[1] * k);
      if (!(b.flags & PGB_BOX_BDY_INTERIOR) && !b.cmask_bdy[p]) continue;
      if (PROG && lv.nvar > 1) {
         acc += relax_vars(b, lv.nvar, p, dim);
         continue;
      }
      double uc = u[p], s = src[p];
      double res = op64<PROG>(pde, b, p, lap64(b, u, p, dim), uc, s) - rhs[p];
      double jac = jac64<PROG>(pde, b, p, uc, s);
      u[p] = uc - res / jac;
      acc += res * res;
   }
   acc = block_sum(acc, sm);
   if (threadIdx.x == 0 && threadIdx.y == 0) sc.partial[pass * lv.nrtiles + blockIdx.x] = acc;
   if (pass == 1 && last_block(sc, &flag))
      finalize_norm(boxes, lv, lv.rtile_start, lv.nrtiles, 2, sc, norm_out, trace, 0, sm);
}

extern "C" int pgb_k_relax(const pgb_dbox *boxes, pgb_dlevel lv, int pde, pgb_scratch sc,
                           double *norm_out, pgb_trace *trace, void *stream)
{
   dim3 blk(PGB_TX, PGB_TY);
   cudaStream_t st = (cudaStream_t)stream;
   if (lv.nrtiles == 0) return 0;
   OPLAUNCH(k_relax, pde, lv.nrtiles, blk, 0, st, boxes, lv, pde, 0, sc, norm_out, trace);
   LAUNCHED(1);
   OPLAUNCH(k_relax, pde, lv.nrtiles, blk, 0, st, boxes, lv, pde, 1, sc, norm_out, trace);
   LAUNCHED(1);
   return check("relax");
}

/* ------------------------------------------------------------- residual -- */
/* residual (num.f:129-161): res = L[u] - rhs where cmask is ON */
template <bool PROG>
__global__ void __launch_bounds__(NT) k_residual(const pgb_dbox *boxes, pgb_dlevel lv, int pde,
                                                 pgb_scratch sc, double *norm_out,
                                                 pgb_trace *trace)
{
   __shared__ double sm[32];
   __shared__ int flag;
   const pgb_tile tl = lv.tiles[blockIdx.x];
   const pgb_dbox b = boxes[tl.box];
   const int dim = lv.dim;
   const double *u = b.f[PGB_F_U], *rhs = b.f[PGB_F_RHS], *src = b.f[PGB_F_SRC];
   double *res = b.f[PGB_F_RES];
   double acc = 0;
   int i = tl.i0 + threadIdx.x, j = tl.j0 + threadIdx.y;
   int kz = dim == 3 ? lv.tz : 1;
   for (int kk = 0; kk < kz; kk++) {
      int k = tl.k0 + kk;
      if (!interior(b, i, j, k, dim)) continue;
      long p = i + (long)b.n[0] * (j + (long)b.n[1] * k);
      if (!(b.flags & PGB_BOX_BDY_INTERIOR) && !b.cmask_bdy[p]) continue;
      if (PROG && lv.nvar > 1) {
         acc += residual_vars(b, lv.nvar, p, dim);
         continue;
      }
      double r = op64<PROG>(pde, b, p, lap64(b, u, p, dim), u[p], src[p]) - rhs[p];
      res[p] = r;
      acc += r * r;
   }
   acc = block_sum(acc, sm);
   if (threadIdx.x == 0 && threadIdx.y == 0) sc.partial[blockIdx.x] = acc;
   if (last_block(sc, &flag))
      finalize_norm(boxes, lv, lv.tile_start, lv.ntiles, 1, sc, norm_out, trace, 1, sm);
}

extern "C" int pgb_k_residual(const pgb_dbox *boxes, pgb_dlevel lv, int pde, pgb_scratch sc,
                              double *norm_out, pgb_trace *trace, void *stream)
{
   if (lv.ntiles == 0) return 0;
   OPLAUNCH(k_residual, pde, lv.ntiles, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream, boxes, lv, pde, sc,
            norm_out, trace);
   LAUNCHED(1);
   return check("residual");
}

/* ------------------------------------------------ pointwise level passes -- */
#define FOR_TILE_POINTS(...) FOR_TILE_POINTS_IN(lv.tiles, __VA_ARGS__)
#define FOR_TILE_POINTS_IN(list, ...)                                                \
   const pgb_tile tl = (list)[blockIdx.x];                                           \
   const pgb_dbox b = boxes[tl.box];                                                 \
   int i = tl.i0 + threadIdx.x, j = tl.j0 + threadIdx.y;                              \
   int kz = lv.dim == 3 ? lv.tz : 1;                                                \
   if (i < b.n[0] && j < b.n[1])                                                     \
      _Pragma("unroll") for (int kk = 0; kk < PGB_TZ; kk++) {                        \
         int k = tl.k0 + kk;                                                         \
         if (kk >= kz || k >= b.n[2]) continue;                                      \
         long p = i + (long)b.n[0] * (j + (long)b.n[1] * k);                         \
         __VA_ARGS__                                                                 \
      }

__global__ void __launch_bounds__(NT) k_clear(const pgb_dbox *boxes, pgb_dlevel lv, int mask)
{
   clear_b(hw_blk(), boxes, lv, mask);
}

/* app_L_op (num.f:85-123, lop = L[u] at interior cmask-child points) fused
 * with compute_MG_rhs (amrd/mg.c:271-314): rhs = cmask ? -res*w0_r + lop : 0,
 * then lop = u, on the level's cover tiles (every child-covered point lies in
 * one; elsewhere rhs keeps the 0 pgb_prepare wrote and lop is never read). */
template <bool PROG>
__global__ void __launch_bounds__(NT) k_lop_rhs(const pgb_dbox *boxes, pgb_dlevel lv, int pde,
                                                double w0_r)
{
   FOR_TILE_POINTS_IN(lv.ctiles, {
      const int cm = b.cmask_child[p];
      if (PROG && lv.nvar > 1) {   /* every variable from the same values of all */
         double uv[PGB_NVAR_MAX], lv_[PGB_NVAR_MAX];
         const pgb_srcv sv = pgb_load_src(b.op->nsrc, b, p, b.f[PGB_F_SRC][p]);
         const bool in = cm && interior(b, i, j, k, lv.dim);
         load_vars(b, lv.nvar, p, uv);
         for (int v = 0; v < lv.nvar; v++)
            lv_[v] = in ? pgb_prog_Lv(b, v, lap64(b, b.f[PGB_FV(v, PGB_F_U)], p, lv.dim), uv, sv) : 0.0;
         for (int v = 0; v < lv.nvar; v++) {
            b.f[PGB_FV(v, PGB_F_RHS)][p] = cm ? -b.f[PGB_FV(v, PGB_F_RES)][p] * w0_r + lv_[v] : 0.0;
            b.f[PGB_FV(v, PGB_F_LOP)][p] = uv[v];
         }
      } else {
         const double *u = b.f[PGB_F_U];
         double lopv = 0;
         if (cm && interior(b, i, j, k, lv.dim))
            lopv = op64<PROG>(pde, b, p, lap64(b, u, p, lv.dim), u[p], b.f[PGB_F_SRC][p]);
         b.f[PGB_F_RHS][p] = cm ? -b.f[PGB_F_RES][p] * w0_r + lopv : 0.0;
         b.f[PGB_F_LOP][p] = u[p];
      }
   })
}

/* compute_cgc first half (amrd/mg.c:332-341): res = (f - lop)/w0_i, on the
 * tiles the interpolation to the finer level reads */
__global__ void __launch_bounds__(NT) k_cgc_coarse(const pgb_dbox *boxes, pgb_dlevel lv,
                                                   double w0_i)
{
   FOR_TILE_POINTS_IN(lv.ctiles, {
      for (int v = 0; v < lv.nvar; v++)
         b.f[PGB_FV(v, PGB_F_RES)][p] = (b.f[PGB_FV(v, PGB_F_U)][p] - b.f[PGB_FV(v, PGB_F_LOP)][p]) / w0_i;
   })
}

/* compute_cgc second half (amrd/mg.c:345-354): f += res */
__global__ void __launch_bounds__(NT) k_add_res(const pgb_dbox *boxes, pgb_dlevel lv)
{
   FOR_TILE_POINTS({
      for (int v = 0; v < lv.nvar; v++) b.f[PGB_FV(v, PGB_F_U)][p] += b.f[PGB_FV(v, PGB_F_RES)][p];
   })
}

extern "C" int pgb_k_clear(const pgb_dbox *boxes, pgb_dlevel lv, int mask, void *stream)
{
   if (!lv.ntiles) return 0;
   if (pgb_tail_recording()) return tail_note(pgb_tail_add_clear(lv, mask), "clear");
   k_clear<<<lv.ntiles, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream>>>(boxes, lv, mask);
   LAUNCHED(1);
   return check("clear");
}
extern "C" int pgb_k_lop_rhs(const pgb_dbox *boxes, pgb_dlevel lv, int pde, double w0_r,
                             void *stream)
{
   if (!lv.nctiles) return 0;
   OPLAUNCH(k_lop_rhs, pde, lv.nctiles, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream, boxes, lv, pde, w0_r);
   LAUNCHED(1);
   return check("lop_rhs");
}
extern "C" int pgb_k_cgc_coarse(const pgb_dbox *boxes, pgb_dlevel lv, double w0_i, void *stream)
{
   if (!lv.nctiles) return 0;
   k_cgc_coarse<<<lv.nctiles, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream>>>(boxes, lv, w0_i);
   LAUNCHED(1);
   return check("cgc_coarse");
}
extern "C" int pgb_k_add_res(const pgb_dbox *boxes, pgb_dlevel lv, void *stream)
{
   if (!lv.ntiles) return 0;
   k_add_res<<<lv.ntiles, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream>>>(boxes, lv);
   LAUNCHED(1);
   return check("add_res");
}

/* --------------------------------------------------------- op-list passes -- */
/* dmcopy3d with unit strides (src/m_util_r8.f:20-50) */
__global__ void k_copy(const pgb_dbox *boxes, const pgb_copy_op *ops, int field)
{
   const pgb_copy_op o = ops[blockIdx.z];
   const pgb_dbox &s = boxes[o.src_box];
   const pgb_dbox &d = boxes[o.dst_box];
   OP_PLANES(o.ni, o.nj, o.nk, {
      d.f[field][lin(d, o.i2 + a, o.j2 + bb, o.k2 + c)] = s.f[field][lin(s, o.i1 + a, o.j1 + bb, o.k1 + c)];
   })
}

/* local_transfer delta = +1 (restrict_b in pgb_weights.cuh) */
__global__ void k_restrict(const pgb_dbox *boxes, const pgb_restrict_op *ops, int field_mask, int res32)
{
   restrict_b(hw_blk(), boxes, ops, field_mask, res32);
}

/* (j*1.0)/irho; for the ratio 2 of every MG hierarchy, the exact product j*0.5 */
__device__ __forceinline__ double frac_rho(int j, int irho)
{
   return irho == 2 ? j * 0.5 : (j * 1.0) / irho;
}

/* one axis of dminterp3d's window (src/m_util_r8.f:65-144, 332-360): the
 * anchors and weights of window point t; n = 1 means a copied anchor */
__device__ __forceinline__ int stencil(int t, int irho, int nanch, int ord, int *a, double *cf)
{
   const int m = irho == 2 ? t >> 1 : t / irho, j = t - m * irho;
   if (j == 0) {
      a[0] = m;
      return 1;
   }
   if (ord == 2 || nanch < 4) {
      double sg = frac_rho(j, irho);
      cf[0] = 1 - sg;
      cf[1] = sg;
      a[0] = m;
      a[1] = m + 1;
      return 2;
   }
   double sg;
   int base;
   if (m == 0) {                 /* left end: i1 <= s1 always holds for the window */
      sg = frac_rho(j, irho);
      base = 0;
   } else if (m == nanch - 2) {  /* right end: (i1+n*s1) > (n1-2*s1) always holds */
      sg = 2.0 + frac_rho(j, irho);
      base = nanch - 4;
   } else {
      sg = 1.0 + frac_rho(j, irho);
      base = m - 1;
   }
   const double HALF = 0.5, MHALF = -0.5;
   const double SIXTH = 0.16666666666666667, MSIXTH = -0.16666666666666667;
   cf[0] = MSIXTH * (sg - 1.0) * (sg - 2.0) * (sg - 3.0);
   cf[1] = HALF * sg * (sg - 2.0) * (sg - 3.0);
   cf[2] = MHALF * sg * (sg - 1.0) * (sg - 3.0);
   cf[3] = SIXTH * sg * (sg - 1.0) * (sg - 2.0);
   for (int q = 0; q < 4; q++) a[q] = base + q;
   return 4;
}

/* sum c[0]*v[0] + c[1]*v[1] + ... left to right (Fortran order) */
__device__ __forceinline__ double wsum(int n, const double *c, const double *v)
{
   if (n == 1) return v[0];
   double r = c[0] * v[0] + c[1] * v[1];
   if (n == 4) {
      r = r + c[2] * v[2];
      r = r + c[3] * v[3];
   }
   return r;
}

/* local_transfer delta = -1 (src/transfer.c:1085-1116): interpolate the
 * coarse window (i-lines, then j-lines, then k-lines, as dminterp3d does)
 * and write the requested fine segment */
__global__ void k_interp(const pgb_dbox *boxes, const pgb_interp_op *ops, int field, int dim)
{
   const pgb_interp_op o = ops[blockIdx.z];
   const pgb_dbox &s = boxes[o.src_box];
   const pgb_dbox &d = boxes[o.dst_box];
   const double *u = s.f[field];
   for (int row = blockIdx.y; row < o.njb * o.nkb; row += gridDim.y) {
      const int bb = row % o.njb, c = row / o.njb;
      const int ty = o.j2b - 1 + bb, tz = o.k2b - 1 + c;
      int ay[4], az[4];
      double cy[4], cz[4];
      const int ny = stencil(ty, o.irho, o.nji, o.ord, ay, cy);
      const int nz = dim == 3 ? stencil(tz, o.irho, o.nki, o.ord, az, cz) : 1;
      if (dim != 3) az[0] = 0;
      for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < o.nib; a += gridDim.x * blockDim.x) {
         const int tx = o.i2b - 1 + a;
         int ax[4];
         double cx[4];
         const int nx = stencil(tx, o.irho, o.nii, o.ord, ax, cx);
         double kv[4];
         for (int r = 0; r < nz; r++) {
            double jv[4];
            for (int qq = 0; qq < ny; qq++) {
               double iv[4];
               for (int pp = 0; pp < nx; pp++)
                  iv[pp] = u[lin(s, o.i1i + ax[pp], o.j1i + ay[qq], o.k1i + az[r])];
               jv[qq] = wsum(nx, cx, iv);
            }
            kv[r] = wsum(ny, cy, jv);
         }
         d.f[field][lin(d, o.i2 + a, o.j2 + bb, o.k2 + c)] = wsum(nz, cz, kv);
      }
   }
}

extern "C" int pgb_k_copy(const pgb_dbox *boxes, const pgb_plan *p, int field, void *stream)
{
   TAIL_REFUSE("copy");
   const pgb_copy_op *h = (const pgb_copy_op *)p->h_ops, *d = (const pgb_copy_op *)p->d_ops;
   for (int bt = 0; bt < p->nbatch; bt++) {
      const int n = p->batch_start[bt + 1] - p->batch_start[bt];
      for (int c0 = 0; c0 < n; c0 += 65535) {
         const int m = n - c0 < 65535 ? n - c0 : 65535;
         dim3 g;
         plane_grid(h + p->batch_start[bt] + c0, m, g);
         k_copy<<<g, 256, 0, (cudaStream_t)stream>>>(boxes, d + p->batch_start[bt] + c0, field);
         LAUNCHED(1);
      }
   }
   return check("copy");
}

extern "C" int pgb_k_restrict(const pgb_dbox *boxes, const pgb_plan *p, int field_mask, int res32,
                              void *stream)
{
   if (pgb_tail_recording()) return tail_note(pgb_tail_add_restrict(p, field_mask, res32), "restrict");
   const pgb_restrict_op *h = (const pgb_restrict_op *)p->h_ops, *d = (const pgb_restrict_op *)p->d_ops;
   for (int bt = 0; bt < p->nbatch; bt++) {
      const int n = p->batch_start[bt + 1] - p->batch_start[bt];
      for (int c0 = 0; c0 < n; c0 += 65535) {
         const int m = n - c0 < 65535 ? n - c0 : 65535;
         dim3 g;
         plane_grid(h + p->batch_start[bt] + c0, m, g);
         k_restrict<<<g, 256, 0, (cudaStream_t)stream>>>(boxes, d + p->batch_start[bt] + c0, field_mask,
                                                         res32);
         LAUNCHED(1);
      }
   }
   return check("restrict");
}

extern "C" int pgb_k_interp(const pgb_dbox *boxes, const pgb_plan *p, int field, int dim,
                            void *stream)
{
   const pgb_interp_op *h = (const pgb_interp_op *)p->h_ops, *d = (const pgb_interp_op *)p->d_ops;
   for (int bt = 0; bt < p->nbatch; bt++) {
      const int n = p->batch_start[bt + 1] - p->batch_start[bt];
      for (int c0 = 0; c0 < n; c0 += 65535) {
         const int m = n - c0 < 65535 ? n - c0 : 65535;
         dim3 g;
         row_grid(h + p->batch_start[bt] + c0, m, g);
         k_interp<<<g, 128, 0, (cudaStream_t)stream>>>(boxes, d + p->batch_start[bt] + c0, field, dim);
         LAUNCHED(1);
      }
   }
   return check("interp");
}

/* ------------------------------------------------------- coarsest grids -- */
/* The coarsest-grid loop of vcycle (amrd/mg.c:172-190) in one CTA: relax
 * the coarsest boxes (both colours), take the call_rr_app norm, sync them
 * (PAMR_sync(L,0,MGH,1) over coarsest grids only), until res <= ctol or
 * max_citer iterations.
 *
 * Below the rounding floor the iteration often revisits earlier states. A
 * 64-bit hash of the state after each iteration is kept for the last
 * PGB_CHASH iterations; when the current hash equals the one p iterations
 * back, the state is saved and p more iterations are run: if the state then
 * equals the saved one exactly, the iteration is periodic with period p, all
 * norms of the cycle exceed ctol (the loop kept going), and the reference
 * would repeat the cycle until max_citer. The loop then skips a multiple of
 * p iterations and runs the remainder, ending on the same state and norm
 * the reference reaches by iterating. */
#define CT 1024
#define PGB_CHASH 256

__device__ __forceinline__ unsigned long long mix64(unsigned long long z)
{
   z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
   z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
   return z ^ (z >> 31);
}

__device__ unsigned long long block_xor(unsigned long long v, unsigned long long *sm)
{
   int t = threadIdx.x;
   for (int o = 16; o > 0; o >>= 1) v ^= __shfl_down_sync(0xffffffffu, v, o);
   if ((t & 31) == 0) sm[t >> 5] = v;
   __syncthreads();
   if (t < 32) {
      v = (t < (blockDim.x >> 5)) ? sm[t] : 0ull;
      for (int o = 16; o > 0; o >>= 1) v ^= __shfl_down_sync(0xffffffffu, v, o);
      if (t == 0) sm[0] = v;
   }
   __syncthreads();
   v = sm[0];
   __syncthreads();
   return v;
}

template <bool PROG>
__global__ void __launch_bounds__(CT) k_coarsest(const pgb_dbox *boxes, pgb_dlevel lv, int pde,
                                                 const pgb_copy_op *sync_ops, int nsync,
                                                 pgb_coarsest_args a, pgb_trace *trace)
{
   __shared__ double sm[32];
   __shared__ unsigned long long smh[32];
   __shared__ unsigned long long hist[PGB_CHASH];
   __shared__ int s_flag;
   const int t = threadIdx.x, dim = lv.dim;
   double ctol = a.ctol_from_first ? -1.0 : *a.res_dn * a.crtol;
   double res = ctol + 1;
   int iter = a.start_iter, nhist = 0;
   int verify_at = -1, period = 0;
   double *saved = a.snap;
   double res_ck = 1e300;   /* over-relaxed loops: the norm at the last check */
   while (iter < a.max_citer && res > ctol) {
      double lres = 0;
      int first = 1;
      for (int b = 0; b < lv.nbox; b++) {
         const pgb_dbox bx = boxes[lv.box[b]];
         if (!(bx.flags & PGB_BOX_COARSEST)) continue;
         long ni = bx.n[0] - 2, nj = bx.n[1] - 2, nk = dim == 3 ? bx.n[2] - 2 : 1;
         long npts = ni * nj * nk;
         double acc = 0;
         for (int pass = 0; pass < 2; pass++) {
            for (long q = t; q < npts; q += CT) {
               int i = 1 + (int)(q % ni), j = 1 + (int)((q / ni) % nj);
               int k = dim == 3 ? 1 + (int)(q / (ni * nj)) : 0;
               int par = dim == 3 ? ((i + j + k + 3 + pass) & 1) : ((i + j + 2 + pass) & 1);
               if (par) continue;
               long p = i + (long)bx.n[0] * (j + (long)bx.n[1] * k);
               if (!(bx.flags & PGB_BOX_BDY_INTERIOR) && !bx.cmask_bdy[p]) continue;
               if (PROG && lv.nvar > 1) {
                  acc += a.sor ? relax_vars_block(bx, lv.nvar, p, dim, a.omega) : relax_vars(bx, lv.nvar, p, dim);
                  continue;
               }
               double *u = bx.f[PGB_F_U];
               double uc = u[p], s = bx.f[PGB_F_SRC][p];
               double r = op64<PROG>(pde, bx, p, lap64(bx, u, p, dim), uc, s) - bx.f[PGB_F_RHS][p];
               double jac = jac64<PROG>(pde, bx, p, uc, s);
               u[p] = uc - r / jac;
               acc += r * r;
            }
            __syncthreads();
         }
         acc = block_sum(acc, sm);
         if (t == 0) {
            double r = sqrt(acc / bx.count);
            if (first) lres = r;
            lres = (r > lres) ? r : lres;
            first = 0;
            if (trace) {
               int n = trace->n;
               if (n < trace->cap) {
                  pgb_trace_rec rr = {0, lv.level, b, 1, r};
                  trace->rec[n] = rr;
                  trace->n = n + 1;
               } else
                  trace->overflow = 1;
            }
         }
         __syncthreads();
      }
      /* PAMR_sync(L,0,MGH,1) restricted to the coarsest grids */
      for (int o = 0; o < nsync; o++) {
         const pgb_copy_op op = sync_ops[o];
         const pgb_dbox &s = boxes[op.src_box];
         const pgb_dbox &d = boxes[op.dst_box];
         long np = (long)op.ni * op.nj * op.nk;
         for (long q = t; q < np; q += CT) {
            int aa, bb, cc;
            unflat(q, op.ni, op.nj, aa, bb, cc);
            for (int v = 0; v < lv.nvar; v++)
               d.f[PGB_FV(v, PGB_F_U)][lin(d, op.i2 + aa, op.j2 + bb, op.k2 + cc)] =
                  s.f[PGB_FV(v, PGB_F_U)][lin(s, op.i1 + aa, op.j1 + bb, op.k1 + cc)];
         }
         __syncthreads();
      }
      if (t == 0) sm[0] = lres;
      __syncthreads();
      double res_before = res;
      res = sm[0];
      __syncthreads();
      if (ctol < 0) {
         ctol = res * a.crtol;
         res_before = res * 2;
      }
      iter++;
      if (!(iter < a.max_citer && res > ctol)) break;
      if (a.stagnation_exit && iter > a.start_iter + 1) {
         if (!a.sor && res >= res_before) break;
         /* over-relaxed sweeps need not lower the norm every sweep: every
          * 8 sweeps it must have fallen since the last check */
         if (a.sor && (iter - a.start_iter) % 8 == 0) {
            if (res >= res_ck) break;
            res_ck = res;
         }
      }
      if (a.sor) continue;   /* no exact periods to skip outside the FP64 form's loop */

      /* hash of the state; at a verification point compare with the save */
      unsigned long long h = 0;
      if (t == 0) s_flag = 0;
      __syncthreads();
      {
         long off = 0;
         for (int b = 0; b < lv.nbox; b++) {
            const pgb_dbox bx = boxes[lv.box[b]];
            if (!(bx.flags & PGB_BOX_COARSEST)) continue;
            long n = (long)bx.n[0] * bx.n[1] * bx.n[2];
            for (int w = 0; w < lv.nvar; w++)   /* the state: every variable */
               for (long q = t; q < n; q += CT) {
                  const long o = w * a.snap_points + off + q;
                  double v = bx.f[PGB_FV(w, PGB_F_U)][q];
                  unsigned long long bits = (unsigned long long)__double_as_longlong(v);
                  h ^= mix64(bits ^ mix64((unsigned long long)o + 0x9E3779B97F4A7C15ull));
                  if (iter == verify_at && saved[o] != v) s_flag = 1;
               }
            off += n;
         }
      }
      h = block_xor(h, smh);
      if (iter == verify_at) {
         if (!s_flag) {
            /* exact period: skip whole periods, run the remainder */
            int rem = a.max_citer - iter;
            int skip = rem - rem % period;
            if (trace && t == 0 && skip > 0) {
               int n = trace->n;
               if (n < trace->cap) {
                  pgb_trace_rec rr = {2, lv.level, period, skip, 0.0};
                  trace->rec[n] = rr;
                  trace->n = n + 1;
               } else
                  trace->overflow = 1;
            }
            iter += skip;
            nhist = 0;
         }
         verify_at = -1;
      } else if (verify_at < 0) {
         int found = 0;
         int lim = nhist < PGB_CHASH ? nhist : PGB_CHASH;
         for (int p = 1; p <= lim && !found; p++)
            if (hist[(nhist - p) % PGB_CHASH] == h) found = p;
         if (found) {
            long off = 0;
            for (int b = 0; b < lv.nbox; b++) {
               const pgb_dbox bx = boxes[lv.box[b]];
               if (!(bx.flags & PGB_BOX_COARSEST)) continue;
               long n = (long)bx.n[0] * bx.n[1] * bx.n[2];
               for (int w = 0; w < lv.nvar; w++)
                  for (long q = t; q < n; q += CT) saved[w * a.snap_points + off + q] = bx.f[PGB_FV(w, PGB_F_U)][q];
               off += n;
            }
            period = found;
            verify_at = iter + found;
         }
      }
      __syncthreads();
      if (t == 0) hist[nhist % PGB_CHASH] = h;
      nhist++;
      __syncthreads();
   }
   if (t == 0) {
      *a.res_out = res;
      if (a.iters_out) *a.iters_out += iter - a.start_iter;
   }
}

/* The same loop on a cluster of PGB_CL CTAs (one per SM), for coarsest
 * levels without overlapping boxes: GB300's FP64 rate per SM is low enough
 * that one CTA spends ~10 us per sweep of a 9^3 grid. The colour passes are
 * split over the cluster and separated by cluster barriers; every CTA
 * combines the per-CTA partial norms and state hashes through distributed
 * shared memory in the same fixed order, so all CTAs take the same
 * decisions. Each point is relaxed by exactly one CTA, which also hashes,
 * saves and compares that point (nothing else changes during the loop). */
#define PGB_CL 8
#define CLT 512
#define MAXCB 8
template <bool PROG>
__global__ void __cluster_dims__(PGB_CL, 1, 1) __launch_bounds__(CLT)
   k_coarsest_cl(const pgb_dbox *boxes, pgb_dlevel lv, int pde, pgb_coarsest_args a,
                 pgb_trace *trace)
{
   cg::cluster_group cl = cg::this_cluster();
   const int rank = (int)cl.block_rank(), t = threadIdx.x, dim = lv.dim;
   const long gstride = (long)PGB_CL * CLT;
   __shared__ double part[2][MAXCB];
   __shared__ unsigned long long hpart[2];
   __shared__ int fpart[2];
   __shared__ double sm[32];
   __shared__ unsigned long long smh[32];
   __shared__ unsigned long long hist[PGB_CHASH];
   __shared__ double s_res;
   __shared__ unsigned long long s_h;
   __shared__ int s_changed;
   int cb[MAXCB], ncb = 0;
   for (int b = 0; b < lv.nbox && ncb < MAXCB; b++)
      if (boxes[lv.box[b]].flags & PGB_BOX_COARSEST) cb[ncb++] = b;
   double ctol = a.ctol_from_first ? -1.0 : *a.res_dn * a.crtol;
   double res = ctol + 1;
   int iter = a.start_iter, nhist = 0, verify_at = -1, period = 0, it_no = 0;
   double *saved = a.snap;
   while (iter < a.max_citer && res > ctol) {
      const int par = it_no & 1;
      double acc[MAXCB];
      unsigned long long h = 0;
      int diff = 0;
      for (int c = 0; c < ncb; c++) acc[c] = 0;
      for (int pass = 0; pass < 2; pass++) {
         for (int c = 0; c < ncb; c++) {
            const pgb_dbox bx = boxes[lv.box[cb[c]]];
            const long off = a.snap_off[cb[c]];
            long ni = bx.n[0] - 2, nj = bx.n[1] - 2, nk = dim == 3 ? bx.n[2] - 2 : 1;
            long hw = (ni + 1) / 2, nslot = hw * nj * nk;   /* one slot per point of the colour */
            for (long q = (long)t * PGB_CL + rank; q < nslot; q += gstride) {
               int j = 1 + (int)((q / hw) % nj);
               int k = dim == 3 ? 1 + (int)(q / (hw * nj)) : 0;
               int off = dim == 3 ? ((1 + j + k + 3 + pass) & 1) : ((1 + j + 2 + pass) & 1);
               int i = 1 + 2 * (int)(q % hw) + off;
               if (i > ni) continue;
               long p = i + (long)bx.n[0] * (j + (long)bx.n[1] * k);
               if (!(bx.flags & PGB_BOX_BDY_INTERIOR) && !bx.cmask_bdy[p]) continue;
               double *u = bx.f[PGB_F_U];
               double uc = u[p], s = bx.f[PGB_F_SRC][p];
               double r = op64<PROG>(pde, bx, p, lap64(bx, u, p, dim), uc, s) - bx.f[PGB_F_RHS][p];
               double jac = jac64<PROG>(pde, bx, p, uc, s);
               double nu = uc - r / jac;
               u[p] = nu;
               acc[c] += r * r;
               unsigned long long bits = (unsigned long long)__double_as_longlong(nu);
               h ^= mix64(bits ^ mix64((unsigned long long)(off + p) + 0x9E3779B97F4A7C15ull));
               if (verify_at >= 0 && iter + 1 == verify_at && saved[off + p] != nu) diff = 1;
               if (verify_at < 0) saved[off + p] = nu;   /* candidate save, kept if a match is found */
            }
         }
         if (pass == 0) cl.sync();
      }
      /* per-CTA partials */
      for (int c = 0; c < ncb; c++) {
         double v = block_sum(acc[c], sm);
         if (t == 0) part[par][c] = v;
      }
      h = block_xor(h, smh);
      if (t == 0) s_changed = 0;
      __syncthreads();
      if (diff) s_changed = 1;
      __syncthreads();
      if (t == 0) {
         hpart[par] = h;
         fpart[par] = s_changed;
      }
      cl.sync();
      /* combine over the cluster in rank order (identical in every CTA) */
      if (t == 0) {
         double lres = 0;
         unsigned long long hh = 0;
         int ch = 0;
         for (int c = 0; c < ncb; c++) {
            double v = 0;
            for (int rr = 0; rr < PGB_CL; rr++) v += cl.map_shared_rank(&part[par][0], rr)[c];
            const pgb_dbox &bx = boxes[lv.box[cb[c]]];
            double r = sqrt(v / bx.count);
            if (c == 0) lres = r;
            lres = (r > lres) ? r : lres;
            if (trace && rank == 0) {
               int n = trace->n;
               if (n < trace->cap) {
                  pgb_trace_rec rec = {0, lv.level, cb[c], 1, r};
                  trace->rec[n] = rec;
                  trace->n = n + 1;
               } else
                  trace->overflow = 1;
            }
         }
         for (int rr = 0; rr < PGB_CL; rr++) {
            hh ^= *cl.map_shared_rank(&hpart[par], rr);
            ch |= *cl.map_shared_rank(&fpart[par], rr);
         }
         s_res = lres;
         s_h = hh;
         s_changed = ch;
      }
      __syncthreads();
      double res_before = res;
      res = s_res;
      h = s_h;
      const int changed = s_changed;
      it_no++;
      if (ctol < 0) {
         ctol = res * a.crtol;
         res_before = res * 2;
      }
      iter++;
      if (!(iter < a.max_citer && res > ctol)) break;
      if (a.stagnation_exit && iter > a.start_iter + 1 && res >= res_before) break;
      if (iter == verify_at) {
         if (!changed) {
            int rem = a.max_citer - iter;
            int skip = rem - rem % period;
            if (trace && rank == 0 && t == 0 && skip > 0) {
               int n = trace->n;
               if (n < trace->cap) {
                  pgb_trace_rec rec = {2, lv.level, period, skip, 0.0};
                  trace->rec[n] = rec;
                  trace->n = n + 1;
               } else
                  trace->overflow = 1;
            }
            iter += skip;
            nhist = 0;
         }
         verify_at = -1;
      } else if (verify_at < 0) {
         int found = 0;
         int lim = nhist < PGB_CHASH ? nhist : PGB_CHASH;
         for (int p = 1; p <= lim && !found; p++)
            if (hist[(nhist - p) % PGB_CHASH] == h) found = p;
         if (found) {   /* this iteration's values were saved above */
            period = found;
            verify_at = iter + found;
         }
      }
      __syncthreads();
      if (t == 0) hist[nhist % PGB_CHASH] = h;
      nhist++;
      __syncthreads();
   }
   cl.sync();
   if (rank == 0 && t == 0) {
      *a.res_out = res;
      if (a.iters_out) *a.iters_out += iter - a.start_iter;
   }
}

/* ---------------------------------------------- coarsest grids, on chip -- */


/* The coarsest-grid loop with the whole coarsest level (u, rhs, source and
 * the saved state of the cycle check) held in shared memory: below the
 * rounding floor the loop is latency bound, and keeping the grid on chip
 * removes the global-memory round trips from every sweep. Same iteration,
 * same cycle skip and same results as k_coarsest. */
#define CS_MAXB 16
template <bool PROG>
__global__ void __launch_bounds__(CT) k_coarsest_smem(const pgb_dbox *boxes, pgb_dlevel lv, int pde,
                                                      const pgb_copy_op *sync_ops, int nsync,
                                                      pgb_coarsest_args a, pgb_trace *trace)
{
   extern __shared__ double dsm[];
   __shared__ double sm[32];
   __shared__ unsigned long long smh[32];
   __shared__ unsigned long long hist[PGB_CHASH];
   __shared__ int s_flag;
   __shared__ int cb[CS_MAXB], ncb_s;
   __shared__ long coff[CS_MAXB + 1];
   const int t = threadIdx.x, dim = lv.dim;
   if (t == 0) {
      int n = 0;
      long o = 0;
      for (int b = 0; b < lv.nbox && n < CS_MAXB; b++) {
         const pgb_dbox &bx = boxes[lv.box[b]];
         if (!(bx.flags & PGB_BOX_COARSEST)) continue;
         cb[n] = b;
         coff[n] = o;
         o += (long)bx.n[0] * bx.n[1] * bx.n[2];
         n++;
      }
      coff[n] = o;
      ncb_s = n;
   }
   __syncthreads();
   const int ncb = ncb_s;
   const long tot = coff[ncb];
   double *su = dsm, *srhs = dsm + tot, *ssrc = dsm + 2 * tot, *ssave = dsm + 3 * tot;
   for (int c = 0; c < ncb; c++) {
      const pgb_dbox &bx = boxes[lv.box[cb[c]]];
      long n = (long)bx.n[0] * bx.n[1] * bx.n[2];
      for (long q = t; q < n; q += CT) {
         su[coff[c] + q] = bx.f[PGB_F_U][q];
         srhs[coff[c] + q] = bx.f[PGB_F_RHS][q];
         ssrc[coff[c] + q] = bx.f[PGB_F_SRC][q];
      }
   }
   __syncthreads();
   double ctol = a.ctol_from_first ? -1.0 : *a.res_dn * a.crtol;
   double res = ctol + 1;
   int iter = a.start_iter, nhist = 0, verify_at = -1, period = 0;
   while (iter < a.max_citer && res > ctol) {
      double lres = 0;
      for (int c = 0; c < ncb; c++) {
         const pgb_dbox bx = boxes[lv.box[cb[c]]];
         double *u = su + coff[c];
         const double *rhs = srhs + coff[c], *src = ssrc + coff[c];
         const long sy = bx.n[0], sz = (long)bx.n[0] * bx.n[1];
         long ni = bx.n[0] - 2, nj = bx.n[1] - 2, nk = dim == 3 ? bx.n[2] - 2 : 1;
         long hw = (ni + 1) / 2, nslot = hw * nj * nk;   /* one slot per point of the colour */
         double acc = 0;
         for (int pass = 0; pass < 2; pass++) {
            for (long q = t; q < nslot; q += CT) {
               int j = 1 + (int)((q / hw) % nj);
               int k = dim == 3 ? 1 + (int)(q / (hw * nj)) : 0;
               int off = dim == 3 ? ((1 + j + k + 3 + pass) & 1) : ((1 + j + 2 + pass) & 1);
               int i = 1 + 2 * (int)(q % hw) + off;
               if (i > ni) continue;
               long p = i + sy * j + sz * k;
               if (!(bx.flags & PGB_BOX_BDY_INTERIOR) && !bx.cmask_bdy[p]) continue;
               double uc = u[p], s = src[p];
               double r = op64<PROG>(pde, bx, p, lap64(bx, u, p, dim), uc, s) - rhs[p];
               double jac = jac64<PROG>(pde, bx, p, uc, s);
               u[p] = uc - r / jac;
               acc += r * r;
            }
            __syncthreads();
         }
         acc = block_sum(acc, sm);
         if (t == 0) {
            double r = sqrt(acc / bx.count);
            if (c == 0) lres = r;
            lres = (r > lres) ? r : lres;
            if (trace) {
               int n = trace->n;
               if (n < trace->cap) {
                  pgb_trace_rec rr = {0, lv.level, cb[c], 1, r};
                  trace->rec[n] = rr;
                  trace->n = n + 1;
               } else
                  trace->overflow = 1;
            }
         }
      }
      for (int o = 0; o < nsync; o++) {   /* PAMR_sync(L,0,MGH,1) over the coarsest grids */
         const pgb_copy_op op = sync_ops[o];
         int cs = -1, cd = -1;
         for (int c = 0; c < ncb; c++) {
            if (lv.box[cb[c]] == op.src_box) cs = c;
            if (lv.box[cb[c]] == op.dst_box) cd = c;
         }
         if (cs < 0 || cd < 0) continue;
         const pgb_dbox &bs = boxes[op.src_box];
         const pgb_dbox &bd = boxes[op.dst_box];
         long np = (long)op.ni * op.nj * op.nk;
         for (long q = t; q < np; q += CT) {
            int aa, bb, cc;
            unflat(q, op.ni, op.nj, aa, bb, cc);
            su[coff[cd] + lin(bd, op.i2 + aa, op.j2 + bb, op.k2 + cc)] =
               su[coff[cs] + lin(bs, op.i1 + aa, op.j1 + bb, op.k1 + cc)];
         }
         __syncthreads();
      }
      if (t == 0) sm[0] = lres;
      __syncthreads();
      double res_before = res;
      res = sm[0];
      __syncthreads();
      if (ctol < 0) {
         ctol = res * a.crtol;
         res_before = res * 2;
      }
      iter++;
      if (!(iter < a.max_citer && res > ctol)) break;
      if (a.stagnation_exit && iter > a.start_iter + 1 && res >= res_before) break;
      /* hash of the state; compare with the saved state at a verification point */
      unsigned long long h = 0;
      if (t == 0) s_flag = 0;
      __syncthreads();
      for (long q = t; q < tot; q += CT) {
         double v = su[q];
         unsigned long long bits = (unsigned long long)__double_as_longlong(v);
         h ^= mix64(bits ^ mix64((unsigned long long)q + 0x9E3779B97F4A7C15ull));
         if (iter == verify_at && ssave[q] != v) s_flag = 1;
      }
      h = block_xor(h, smh);
      if (iter == verify_at) {
         if (!s_flag) {
            int rem = a.max_citer - iter;
            int skip = rem - rem % period;
            if (trace && t == 0 && skip > 0) {
               int n = trace->n;
               if (n < trace->cap) {
                  pgb_trace_rec rr = {2, lv.level, period, skip, 0.0};
                  trace->rec[n] = rr;
                  trace->n = n + 1;
               } else
                  trace->overflow = 1;
            }
            iter += skip;
            nhist = 0;
         }
         verify_at = -1;
      } else if (verify_at < 0) {
         int found = 0;
         int lim = nhist < PGB_CHASH ? nhist : PGB_CHASH;
         for (int p = 1; p <= lim && !found; p++)
            if (hist[(nhist - p) % PGB_CHASH] == h) found = p;
         if (found) {
            for (long q = t; q < tot; q += CT) ssave[q] = su[q];
            period = found;
            verify_at = iter + found;
         }
      }
      __syncthreads();
      if (t == 0) hist[nhist % PGB_CHASH] = h;
      nhist++;
      __syncthreads();
   }
   for (int c = 0; c < ncb; c++) {
      const pgb_dbox &bx = boxes[lv.box[cb[c]]];
      long n = (long)bx.n[0] * bx.n[1] * bx.n[2];
      for (long q = t; q < n; q += CT) bx.f[PGB_F_U][q] = su[coff[c] + q];
   }
   if (t == 0) {
      *a.res_out = res;
      if (a.iters_out) *a.iters_out += iter - a.start_iter;
   }
}

extern "C" int pgb_k_coarsest(const pgb_dbox *boxes, pgb_dlevel lv, int pde, const pgb_plan *sync,
                              pgb_coarsest_args a, pgb_trace *trace, void *stream)
{
   TAIL_REFUSE("coarsest");
   size_t smem = (size_t)a.smem_points * 4 * sizeof(double);
   const char *force = getenv("PGB_COARSEST_KERNEL");   /* smem | cluster | single (experiments) */
   int want_smem = (!force || !strcmp(force, "smem")) && lv.nvar == 1;
   int want_cl = (!force || !strcmp(force, "cluster")) && lv.nvar == 1;   /* one variable only */
   if (want_smem && a.smem_points > 0 && a.ncoarse <= CS_MAXB && smem <= 200 * 1024) {
      static int attr_set = 0;
      if (!attr_set) {
         cudaFuncSetAttribute(k_coarsest_smem<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
         cudaFuncSetAttribute(k_coarsest_smem<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
         attr_set = 1;
      }
      OPLAUNCH(k_coarsest_smem, pde, 1, CT, smem, (cudaStream_t)stream, boxes, lv, pde,
               (const pgb_copy_op *)sync->d_ops, sync->nops, a, trace);
      LAUNCHED(1);
   } else if (want_cl && sync->nops == 0 && lv.nbox <= MAXCB) {
      OPLAUNCH(k_coarsest_cl, pde, PGB_CL, CLT, 0, (cudaStream_t)stream, boxes, lv, pde, a, trace);
      LAUNCHED(1);
   } else {
      OPLAUNCH(k_coarsest, pde, 1, CT, 0, (cudaStream_t)stream, boxes, lv, pde, (const pgb_copy_op *)sync->d_ops,
               sync->nops, a, trace);
      LAUNCHED(1);
   }
   return check("coarsest");
}

__global__ void k_fill(double *p, long n, double v)
{
   for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
      p[i] = v;
}

extern "C" int pgb_k_fill(double *p, long n, double v, void *stream)
{
   long g = (n + 255) / 256;
   if (g > 4096) g = 4096;
   if (g < 1) g = 1;
   k_fill<<<(int)g, 256, 0, (cudaStream_t)stream>>>(p, n, v);
   LAUNCHED(1);
   return check("fill");
}

/* --------------------------------------- m_util_r8 on device arrays (ABI) -- */
/* Same argument meaning as src/m_util_r8.f; out-of-range segments are a
 * silent no-op there and here. */
typedef struct {
   int nx1, ny1, nz1, nx2, ny2, nz2, i1, j1, k1, i2, j2, k2, ni, nj, nk;
   int si1, sj1, sk1, si2, sj2, sk2;
} mu_args;

static bool mu_in_range(const mu_args &a)
{
   if (a.i1 < 1 || (a.i1 + (a.ni - 1) * a.si1) > a.nx1) return false;
   if (a.i2 < 1 || (a.i2 + (a.ni - 1) * a.si2) > a.nx2) return false;
   if (a.j1 < 1 || (a.j1 + (a.nj - 1) * a.sj1) > a.ny1) return false;
   if (a.j2 < 1 || (a.j2 + (a.nj - 1) * a.sj2) > a.ny2) return false;
   if (a.k1 < 1 || (a.k1 + (a.nk - 1) * a.sk1) > a.nz1) return false;
   if (a.k2 < 1 || (a.k2 + (a.nk - 1) * a.sk2) > a.nz2) return false;
   return true;
}

/* kind 1 copy (dmcopy3d), 2 half weight (dmhwr3d), 3 full weight (dmfwr3d) */
__global__ void k_mutil(const double *u1, double *u2, mu_args a, int kind)
{
   long npts = (long)a.ni * a.nj * a.nk;
   for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < npts;
        q += (long)gridDim.x * blockDim.x) {
      int i, j, k;
      unflat(q, a.ni, a.nj, i, j, k);
      int i0 = a.i1 + i * a.si1, j0 = a.j1 + j * a.sj1, k0 = a.k1 + k * a.sk1;
      long pd = (a.i2 + i * a.si2 - 1) + (long)a.nx2 * ((a.j2 + j * a.sj2 - 1) + (long)a.ny2 * (a.k2 + k * a.sk2 - 1));
      double v;
      if (kind == 1) v = u1[(i0 - 1) + (long)a.nx1 * ((j0 - 1) + (long)a.ny1 * (k0 - 1))];
      else if (kind == 2) v = hwr(u1, a.nx1, a.ny1, a.nz1, i0, j0, k0);
      else v = fwr(u1, a.nx1, a.ny1, a.nz1, i0, j0, k0);
      u2[pd] = v;
   }
}

static int mutil_launch(const double *u1, double *u2, mu_args a, int kind, void *stream)
{
   if (!mu_in_range(a)) return 0;
   long npts = (long)a.ni * a.nj * a.nk;
   long g = (npts + 255) / 256;
   if (g > 4096) g = 4096;
   if (g < 1) return 0;
   k_mutil<<<(int)g, 256, 0, (cudaStream_t)stream>>>(u1, u2, a, kind);
   LAUNCHED(1);
   if (check("m_util_r8")) {
      pgb_note_error(g_err);
      return 11;
   }
   return 0;
}

#define MU_ARGS                                                                          \
   mu_args a = {nx1, ny1, nz1, nx2, ny2, nz2, i1, j1, k1, i2, j2, k2, ni, nj, nk,     \
                si1, sj1, sk1, si2, sj2, sk2};
#define MU_SIG                                                                           \
   const double *u1, double *u2, int nx1, int ny1, int nz1, int nx2, int ny2, int nz2, \
      int i1, int j1, int k1, int i2, int j2, int k2, int ni, int nj, int nk, int si1,  \
      int sj1, int sk1, int si2, int sj2, int sk2, void *stream

extern "C" int pgb_dmcopy3d(MU_SIG) { MU_ARGS return mutil_launch(u1, u2, a, 1, stream); }
extern "C" int pgb_dmhwr3d(MU_SIG) { MU_ARGS return mutil_launch(u1, u2, a, 2, stream); }
extern "C" int pgb_dmfwr3d(MU_SIG) { MU_ARGS return mutil_launch(u1, u2, a, 3, stream); }

/* dminterp3d (src/m_util_r8.f:473-637), do_ex = 0, on a segment of u2.
 * Cubic lines use one-sided stencils at a segment end only where the
 * Fortran does (left: start <= rho, right: start + n*rho > N - 2*rho);
 * segments whose cubic lines would take interior stencils reaching outside
 * the segment are rejected. */
typedef struct {
   int nx1, ny1, nz1, nx2, ny2, nz2, i1, j1, k1, i2, j2, k2, ni, nj, nk, si1, sj1, sk1;
   int irho, jrho, krho, ord, dim;
} mi_args;

__device__ __forceinline__ int mi_stencil(int t, int rho, int n, int ord, int *a, double *cf)
{
   return stencil(t, rho, n, ord, a, cf);
}

__global__ void k_minterp(const double *u1, double *u2, mi_args a)
{
   long ex = (long)(a.ni - 1) * a.irho + 1, ey = (long)(a.nj - 1) * a.jrho + 1;
   long ez = a.dim == 3 ? (long)(a.nk - 1) * a.krho + 1 : 1;
   long npts = ex * ey * ez;
   for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < npts;
        q += (long)gridDim.x * blockDim.x) {
      int tx = (int)(q % ex), ty = (int)((q / ex) % ey), tz = (int)(q / (ex * ey));
      int ax[4], ay[4], az[4];
      double cx[4], cy[4], cz[4];
      int nx = mi_stencil(tx, a.irho, a.ni, a.ord, ax, cx);
      int ny = mi_stencil(ty, a.jrho, a.nj, a.ord, ay, cy);
      int nz = a.dim == 3 ? mi_stencil(tz, a.krho, a.nk, a.ord, az, cz) : 1;
      if (a.dim != 3) az[0] = 0;
      double kv[4];
      for (int r = 0; r < nz; r++) {
         double jv[4];
         for (int qq = 0; qq < ny; qq++) {
            double iv[4];
            for (int pp = 0; pp < nx; pp++) {
               int ci = a.i1 + ax[pp] * a.si1, cj = a.j1 + ay[qq] * a.sj1, ck = a.k1 + az[r] * a.sk1;
               iv[pp] = u1[(ci - 1) + (long)a.nx1 * ((cj - 1) + (long)a.ny1 * (ck - 1))];
            }
            jv[qq] = wsum(nx, cx, iv);
         }
         kv[r] = wsum(ny, cy, jv);
      }
      long pd = (a.i2 + tx - 1) + (long)a.nx2 * ((a.j2 + ty - 1) + (long)a.ny2 * (a.k2 + tz - 1));
      u2[pd] = wsum(nz, cz, kv);
   }
}

extern "C" int pgb_dminterp3d(const double *u1, double *u2, int nx1, int ny1, int nz1, int nx2,
                              int ny2, int nz2, int i1, int j1, int k1, int i2, int j2, int k2,
                              int ni, int nj, int nk, int si1, int sj1, int sk1, int irho, int jrho,
                              int krho, int ord, void *stream)
{
   mi_args a = {nx1, ny1, nz1, nx2, ny2, nz2, i1, j1, k1, i2, j2, k2, ni, nj, nk,
                si1, sj1, sk1, irho, jrho, krho, ord, nz2 > 1 || nk > 1 ? 3 : 2};
   if (i1 < 1 || (i1 + ni - 1) * si1 > nx1) return 0;
   if (i2 < 1 || (i2 + (ni - 1) * irho) > nx2) return 0;
   if (j1 < 1 || (j1 + nj - 1) * sj1 > ny1) return 0;
   if (j2 < 1 || (j2 + (nj - 1) * jrho) > ny2) return 0;
   if (k1 < 1 || (k1 + nk - 1) * sk1 > nz1) return 0;
   if (k2 < 1 || (k2 + (nk - 1) * krho) > nz2) return 0;
   if (ord != 2 && ord != 4) {
      snprintf(g_err, sizeof(g_err), "dminterp3d: only ord=2,4 supported");
      pgb_note_error(g_err);
      return 12;
   }
   if (ord == 4) {
      int st[3] = {i2, j2, k2}, n[3] = {ni, nj, nk}, r[3] = {irho, jrho, krho}, N[3] = {nx2, ny2, nz2};
      for (int d = 0; d < 3; d++)
         if (n[d] >= 4 && !(st[d] <= r[d] && st[d] + n[d] * r[d] > N[d] - 2 * r[d])) {
            snprintf(g_err, sizeof(g_err),
                     "dminterp3d: cubic segment needs data outside it (unsupported)");
            pgb_note_error(g_err);
            return 12;
         }
   }
   if (nj == 1 && nk == 1) a.dim = 2;
   long npts = ((long)(ni - 1) * irho + 1) * ((long)(nj - 1) * jrho + 1) *
               (a.dim == 3 ? (long)(nk - 1) * krho + 1 : 1);
   long g = (npts + 255) / 256;
   if (g > 4096) g = 4096;
   if (g < 1) return 0;
   k_minterp<<<(int)g, 256, 0, (cudaStream_t)stream>>>(u1, u2, a);
   LAUNCHED(1);
   if (check("dminterp3d")) {
      pgb_note_error(g_err);
      return 11;
   }
   return 0;
}
