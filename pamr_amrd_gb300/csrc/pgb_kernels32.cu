/*
 * Mixed-precision kernels of libpamr_gb300 (sm_103a): FP32 smoothing and
 * FP32 prolongation inside FP64 defect correction.
 *
 * A smoothing block of the FAS V-cycle (MG_pre_swp or MG_pst_swp sweeps of
 * amrd/mg.c:135-141, 161-167) becomes
 *     d = rhs - L[u]                       (FP64 defect, stored as FP32)
 *     e = 0; sweeps of red-black GS on L'(u) e = d   (FP32)
 *     u = u + e                            (FP64 update)
 * For a linear operator the FP32 sweeps produce, up to FP32 rounding of the
 * correction, exactly the correction the FP64 sweeps would; for the
 * nonlinear conformal factor they are the linearised (Newton) sweeps. The
 * coarse-grid correction (f - lop)/w0 is computed in FP64 and interpolated
 * in FP32 (same nested line order as dminterp3d; FP64 on box boundaries)
 * before the FP64 add. The
 * V-cycle keeps every FP64 piece of the reference: residuals, restriction,
 * FAS right-hand sides, coarsest-grid solve and the finest-level norm.
 *
 * Compiled with FMA contraction: nothing here is compared bit for bit.
 */
#include <cuda_runtime.h>
#include <stdio.h>
#include "pgb_dev.h"

static __thread char g_err32[256];
extern "C" unsigned long long pgb_dev_launches(void);
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

#define NT (PGB_TX * PGB_TY)
#define TWO_PI 6.283185307179586
#define TEN_PI 31.41592653589793

enum { W_E = 0, W_D = 1, W_C = 2 };

__device__ __forceinline__ bool interior32(const pgb_dbox &b, int i, int j, int k, int dim)
{
   return i >= 1 && i <= b.n[0] - 2 && j >= 1 && j <= b.n[1] - 2 &&
          (dim == 2 ? k == 0 : (k >= 1 && k <= b.n[2] - 2));
}

/* FP64 defect d = rhs - L[u] and the FP32 Jacobian term c = dL/du - lap part;
 * e = 0. Points outside the relaxed set get d = 0 so e stays 0 there. */
__global__ void __launch_bounds__(NT) k_defect(const pgb_dbox *boxes, pgb_dlevel lv, int pde)
{
   const pgb_tile tl = lv.tiles[blockIdx.x];
   const pgb_dbox b = boxes[tl.box];
   const int dim = lv.dim;
   int i = tl.i0 + threadIdx.x, j = tl.j0 + threadIdx.y;
   if (i >= b.n[0] || j >= b.n[1]) return;
   const double *u = b.f[PGB_F_U], *rhs = b.f[PGB_F_RHS], *src = b.f[PGB_F_SRC];
   const long sy = b.n[0], sz = (long)b.n[0] * b.n[1];
   int kz = dim == 3 ? lv.tz : 1;
   for (int kk = 0; kk < kz; kk++) {
      int k = tl.k0 + kk;
      if (k >= b.n[2]) break;
      long p = i + sy * j + sz * k;
      float d = 0.f, c = 0.f;
      if (interior32(b, i, j, k, dim) && ((b.flags & PGB_BOX_BDY_INTERIOR) || b.cmask_bdy[p])) {
         double uc = u[p], s = src[p];
         double t = (u[p + 1] - 2 * uc + u[p - 1]) * b.idx2[0] +
                    (u[p + sy] - 2 * uc + u[p - sy]) * b.idx2[1];
         if (dim == 3) t += (u[p + sz] - 2 * uc + u[p - sz]) * b.idx2[2];
         double l, dc = 0;
         if (pde == 1) {
            double p2 = uc * uc, p4 = p2 * p2;
            l = t + TWO_PI * s * (p4 * uc);
            dc = TEN_PI * s * p4;
         } else if (pde == 2) {
            l = t - s * uc;
            dc = -s;
         } else
            l = t - s;
         d = (float)(rhs[p] - l);
         c = (float)dc;
      }
      b.w32[W_D][p] = d;
      b.w32[W_C][p] = c;
      b.w32[W_E][p] = 0.f;
   }
}

/* one colour pass of GS on L'(u) e = d, FP32 (parity as num.f:220) */
__global__ void __launch_bounds__(NT) k_relax32(const pgb_dbox *boxes, pgb_dlevel lv, int pass)
{
   const pgb_tile tl = lv.rtiles[blockIdx.x];
   const pgb_dbox b = boxes[tl.box];
   const int dim = lv.dim;
   float *e = b.w32[W_E];
   const float *dd = b.w32[W_D], *cc = b.w32[W_C];
   const long sy = b.n[0], sz = (long)b.n[0] * b.n[1];
   const float ix = (float)b.idx2[0], iy = (float)b.idx2[1], iz = (float)b.idx2[2];
   const float j0 = (float)b.j0;
   int j = tl.j0 + threadIdx.y;
   int kz = dim == 3 ? lv.rtz : 1;
   for (int kk = 0; kk < kz; kk++) {
      int k = tl.k0 + kk;
      int par = dim == 3 ? ((j + k + 1 + pass) & 1) : ((j + pass) & 1);
      int i = tl.i0 + 2 * threadIdx.x + par;
      if (!interior32(b, i, j, k, dim)) continue;
      long p = i + sy * j + sz * k;
      if (!(b.flags & PGB_BOX_BDY_INTERIOR) && !b.cmask_bdy[p]) continue;
      float ec = e[p], c = cc[p];
      float t = (e[p + 1] - 2.f * ec + e[p - 1]) * ix + (e[p + sy] - 2.f * ec + e[p - sy]) * iy;
      if (dim == 3) t += (e[p + sz] - 2.f * ec + e[p - sz]) * iz;
      float r = t + c * ec - dd[p];
      e[p] = ec - r / (j0 + c);
   }
}

/* u += e (FP64 update) */
__global__ void __launch_bounds__(NT) k_update(const pgb_dbox *boxes, pgb_dlevel lv)
{
   const pgb_tile tl = lv.tiles[blockIdx.x];
   const pgb_dbox b = boxes[tl.box];
   int i = tl.i0 + threadIdx.x, j = tl.j0 + threadIdx.y;
   if (i >= b.n[0] || j >= b.n[1]) return;
   int kz = lv.dim == 3 ? lv.tz : 1;
   for (int kk = 0; kk < kz; kk++) {
      int k = tl.k0 + kk;
      if (k >= b.n[2]) break;
      long p = i + (long)b.n[0] * (j + (long)b.n[1] * k);
      b.f[PGB_F_U][p] += (double)b.w32[W_E][p];
   }
}

__device__ __forceinline__ long lin32(const pgb_dbox &b, int i1, int j1, int k1)
{
   return (i1 - 1) + (long)b.n[0] * ((j1 - 1) + (long)b.n[1] * (k1 - 1));
}

/* FP32 copy of the correction along a sync plan (PAMR_sync of e) */
__global__ void k_copy32(const pgb_dbox *boxes, const pgb_copy_op *ops)
{
   const pgb_copy_op o = ops[blockIdx.y];
   long npts = (long)o.ni * o.nj * o.nk;
   const pgb_dbox &s = boxes[o.src_box];
   const pgb_dbox &d = boxes[o.dst_box];
   for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < npts;
        q += (long)gridDim.x * blockDim.x) {
      int a = (int)(q % o.ni), bb = (int)((q / o.ni) % o.nj), c = (int)(q / ((long)o.ni * o.nj));
      d.w32[W_E][lin32(d, o.i2 + a, o.j2 + bb, o.k2 + c)] =
         s.w32[W_E][lin32(s, o.i1 + a, o.j1 + bb, o.k1 + c)];
   }
}

/* window stencil of dminterp3d in FP32 (linear; cubic with one-sided ends) */
__device__ __forceinline__ int stencil32(int t, int irho, int nanch, int ord, int *a, float *cf)
{
   int m = t / irho, j = t - m * irho;
   if (j == 0) {
      a[0] = m;
      return 1;
   }
   if (ord == 2 || nanch < 4) {
      float sg = (float)j / irho;
      cf[0] = 1.f - sg;
      cf[1] = sg;
      a[0] = m;
      a[1] = m + 1;
      return 2;
   }
   float sg;
   int base;
   if (m == 0) {
      sg = (float)j / irho;
      base = 0;
   } else if (m == nanch - 2) {
      sg = 2.f + (float)j / irho;
      base = nanch - 4;
   } else {
      sg = 1.f + (float)j / irho;
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

/* FP64 weights of the same window stencil (used on box-boundary points) */
__device__ __forceinline__ int stencil64m(int t, int irho, int nanch, int ord, int *a, double *cf)
{
   int m = t / irho, j = t - m * irho;
   if (j == 0) {
      a[0] = m;
      return 1;
   }
   if (ord == 2 || nanch < 4) {
      double sg = (double)j / irho;
      cf[0] = 1.0 - sg;
      cf[1] = sg;
      a[0] = m;
      a[1] = m + 1;
      return 2;
   }
   double sg;
   int base;
   if (m == 0) {
      sg = (double)j / irho;
      base = 0;
   } else if (m == nanch - 2) {
      sg = 2.0 + (double)j / irho;
      base = nanch - 4;
   } else {
      sg = 1.0 + (double)j / irho;
      base = m - 1;
   }
   cf[0] = -0.16666666666666667 * (sg - 1.0) * (sg - 2.0) * (sg - 3.0);
   cf[1] = 0.5 * sg * (sg - 2.0) * (sg - 3.0);
   cf[2] = -0.5 * sg * (sg - 1.0) * (sg - 3.0);
   cf[3] = 0.16666666666666667 * sg * (sg - 1.0) * (sg - 2.0);
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

/* coarse-grid correction, interpolation half: fine res = interpolation of
 * coarse res (amrd/mg.c:343), assigned in plan order like the FP64 path.
 * Interior fine points interpolate in FP32 -- the next FP64 defect sees and
 * corrects their rounding -- while points on a fine box's boundary, which no
 * defect covers (their values only change through these corrections),
 * interpolate in FP64. */
__global__ void k_interp_mixed(const pgb_dbox *boxes, const pgb_interp_op *ops, int dim)
{
   const pgb_interp_op o = ops[blockIdx.y];
   long npts = (long)o.nib * o.njb * o.nkb;
   const pgb_dbox &s = boxes[o.src_box];
   const pgb_dbox &d = boxes[o.dst_box];
   const double *u = s.f[PGB_F_RES];
   for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < npts;
        q += (long)gridDim.x * blockDim.x) {
      int a = (int)(q % o.nib), bb = (int)((q / o.nib) % o.njb), c = (int)(q / ((long)o.nib * o.njb));
      int fi = o.i2 + a, fj = o.j2 + bb, fk = o.k2 + c;
      bool edge = fi == 1 || fi == d.n[0] || fj == 1 || fj == d.n[1] ||
                  (dim == 3 && (fk == 1 || fk == d.n[2]));
      int tx = o.i2b - 1 + a, ty = o.j2b - 1 + bb, tz = o.k2b - 1 + c;
      int ax[4], ay[4], az[4];
      double v;
      if (edge) {
         double cx[4], cy[4], cz[4], kv[4];
         int nx = stencil64m(tx, o.irho, o.nii, o.ord, ax, cx);
         int ny = stencil64m(ty, o.irho, o.nji, o.ord, ay, cy);
         int nz = dim == 3 ? stencil64m(tz, o.irho, o.nki, o.ord, az, cz) : 1;
         if (dim != 3) az[0] = 0;
         for (int r = 0; r < nz; r++) {
            double jv[4];
            for (int qq = 0; qq < ny; qq++) {
               double iv[4];
               for (int pp = 0; pp < nx; pp++)
                  iv[pp] = u[lin32(s, o.i1i + ax[pp], o.j1i + ay[qq], o.k1i + az[r])];
               jv[qq] = wsum64m(nx, cx, iv);
            }
            kv[r] = wsum64m(ny, cy, jv);
         }
         v = wsum64m(nz, cz, kv);
      } else {
         float cx[4], cy[4], cz[4], kv[4];
         int nx = stencil32(tx, o.irho, o.nii, o.ord, ax, cx);
         int ny = stencil32(ty, o.irho, o.nji, o.ord, ay, cy);
         int nz = dim == 3 ? stencil32(tz, o.irho, o.nki, o.ord, az, cz) : 1;
         if (dim != 3) az[0] = 0;
         for (int r = 0; r < nz; r++) {
            float jv[4];
            for (int qq = 0; qq < ny; qq++) {
               float iv[4];
               for (int pp = 0; pp < nx; pp++)
                  iv[pp] = (float)u[lin32(s, o.i1i + ax[pp], o.j1i + ay[qq], o.k1i + az[r])];
               jv[qq] = wsum32(nx, cx, iv);
            }
            kv[r] = wsum32(ny, cy, jv);
         }
         v = (double)wsum32(nz, cz, kv);
      }
      d.f[PGB_F_RES][lin32(d, fi, fj, fk)] = v;
   }
}

/* ------------------------------------------------------------ launchers -- */
extern "C" int pgb_k_defect(const pgb_dbox *boxes, pgb_dlevel lv, int pde, void *stream)
{
   if (!lv.ntiles) return 0;
   k_defect<<<lv.ntiles, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream>>>(boxes, lv, pde);
   return check32("defect");
}

extern "C" int pgb_k_relax32(const pgb_dbox *boxes, pgb_dlevel lv, void *stream)
{
   if (!lv.nrtiles) return 0;
   k_relax32<<<lv.nrtiles, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream>>>(boxes, lv, 0);
   if (check32("relax32")) return 1;
   k_relax32<<<lv.nrtiles, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream>>>(boxes, lv, 1);
   return check32("relax32");
}

extern "C" int pgb_k_update(const pgb_dbox *boxes, pgb_dlevel lv, void *stream)
{
   if (!lv.ntiles) return 0;
   k_update<<<lv.ntiles, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream>>>(boxes, lv);
   return check32("update");
}

extern "C" int pgb_k_copy32(const pgb_dbox *boxes, const pgb_plan *p, void *stream)
{
   for (int bt = 0; bt < p->nbatch; bt++) {
      int n = p->batch_start[bt + 1] - p->batch_start[bt];
      int gx = (p->batch_maxpts[bt] + 255) / 256;
      if (gx > 512) gx = 512;
      if (n <= 0 || gx <= 0) continue;
      for (int c0 = 0; c0 < n; c0 += 65535) {
         k_copy32<<<dim3(gx, n - c0 < 65535 ? n - c0 : 65535), 256, 0, (cudaStream_t)stream>>>(
            boxes, (const pgb_copy_op *)p->d_ops + p->batch_start[bt] + c0);
         if (check32("copy32")) return 1;
      }
   }
   return 0;
}

extern "C" int pgb_k_interp_mixed(const pgb_dbox *boxes, const pgb_plan *p, int dim, void *stream)
{
   for (int bt = 0; bt < p->nbatch; bt++) {
      int n = p->batch_start[bt + 1] - p->batch_start[bt];
      int gx = (p->batch_maxpts[bt] + 255) / 256;
      if (gx > 2048) gx = 2048;
      if (n <= 0 || gx <= 0) continue;
      for (int c0 = 0; c0 < n; c0 += 65535) {
         k_interp_mixed<<<dim3(gx, n - c0 < 65535 ? n - c0 : 65535), 256, 0, (cudaStream_t)stream>>>(
            boxes, (const pgb_interp_op *)p->d_ops + p->batch_start[bt] + c0, dim);
         if (check32("interp_mixed")) return 1;
      }
   }
   return 0;
}

/* ---------------------------------------- FP64 passes of the mixed form -- */
/* The mixed form needs FP64 accuracy in its residuals, not the reference's
 * bit pattern: these variants multiply by 1/dx^2 and let the compiler fuse
 * multiply-adds, which roughly halves their FP64 instruction count. */
__device__ __forceinline__ double lapf(const pgb_dbox &b, const double *u, long p, int dim)
{
   long sy = b.n[0], sz = (long)b.n[0] * b.n[1];
   double c = u[p];
   double t = (u[p + 1] - 2 * c + u[p - 1]) * b.idx2[0] + (u[p + sy] - 2 * c + u[p - sy]) * b.idx2[1];
   if (dim == 3) t += (u[p + sz] - 2 * c + u[p - sz]) * b.idx2[2];
   return t;
}

__device__ __forceinline__ double opf(int pde, double t, double u, double s)
{
   if (pde == 1) {
      double p2 = u * u;
      return t + TWO_PI * s * (p2 * p2 * u);
   }
   if (pde == 2) return t - s * u;
   return t - s;
}

__device__ double block_sum32(double v, double *sm)
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
   return v;
}

__global__ void __launch_bounds__(NT) k_residual_fast(const pgb_dbox *boxes, pgb_dlevel lv, int pde,
                                                      pgb_scratch sc, double *norm_out,
                                                      pgb_trace *trace)
{
   __shared__ double sm[32];
   __shared__ int last;
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
      if (!interior32(b, i, j, k, dim)) continue;
      long p = i + (long)b.n[0] * (j + (long)b.n[1] * k);
      if (!(b.flags & PGB_BOX_BDY_INTERIOR) && !b.cmask_bdy[p]) continue;
      double r = opf(pde, lapf(b, u, p, dim), u[p], src[p]) - rhs[p];
      res[p] = r;
      acc += r * r;
   }
   acc = block_sum32(acc, sm);
   if (threadIdx.x == 0 && threadIdx.y == 0) sc.partial[blockIdx.x] = acc;
   __threadfence();
   __syncthreads();
   if (threadIdx.x == 0 && threadIdx.y == 0)
      last = (atomicAdd(sc.counter, 1u) == gridDim.x * gridDim.y - 1);
   __syncthreads();
   if (!last) return;
   /* call_rr_app: per-box RMS, max over boxes */
   int t = threadIdx.x + threadIdx.y * blockDim.x;
   double lres = 0;
   for (int bx = 0; bx < lv.nbox; bx++) {
      double v = 0;
      for (int s = lv.tile_start[bx] + t; s < lv.tile_start[bx + 1]; s += NT) v += __ldcg(&sc.partial[s]);
      v = block_sum32(v, sm);
      if (t == 0) {
         double r = sqrt(v / boxes[lv.box[bx]].count);
         if (bx == 0) lres = r;
         lres = (r > lres) ? r : lres;
         if (trace) {
            int n = trace->n;
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

/* L_op + compute_MG_rhs (amrd/mg.c:271-314) for the mixed form */
__global__ void __launch_bounds__(NT) k_lop_rhs_fast(const pgb_dbox *boxes, pgb_dlevel lv, int pde,
                                                     double w0_r)
{
   const pgb_tile tl = lv.tiles[blockIdx.x];
   const pgb_dbox b = boxes[tl.box];
   int i = tl.i0 + threadIdx.x, j = tl.j0 + threadIdx.y;
   if (i >= b.n[0] || j >= b.n[1]) return;
   const double *u = b.f[PGB_F_U];
   int kz = lv.dim == 3 ? lv.tz : 1;
   for (int kk = 0; kk < kz; kk++) {
      int k = tl.k0 + kk;
      if (k >= b.n[2]) break;
      long p = i + (long)b.n[0] * (j + (long)b.n[1] * k);
      double lopv = 0;
      int cm = b.cmask_child[p];
      if (cm && interior32(b, i, j, k, lv.dim)) lopv = opf(pde, lapf(b, u, p, lv.dim), u[p], b.f[PGB_F_SRC][p]);
      b.f[PGB_F_RHS][p] = cm ? -b.f[PGB_F_RES][p] * w0_r + lopv : 0.0;
      b.f[PGB_F_LOP][p] = u[p];
   }
}

extern "C" int pgb_k_residual_fast(const pgb_dbox *boxes, pgb_dlevel lv, int pde, pgb_scratch sc,
                                   double *norm_out, pgb_trace *trace, void *stream)
{
   if (!lv.ntiles) return 0;
   k_residual_fast<<<lv.ntiles, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream>>>(boxes, lv, pde, sc,
                                                                                  norm_out, trace);
   return check32("residual_fast");
}

extern "C" int pgb_k_lop_rhs_fast(const pgb_dbox *boxes, pgb_dlevel lv, int pde, double w0_r,
                                  void *stream)
{
   if (!lv.ntiles) return 0;
   k_lop_rhs_fast<<<lv.ntiles, dim3(PGB_TX, PGB_TY), 0, (cudaStream_t)stream>>>(boxes, lv, pde, w0_r);
   return check32("lop_rhs_fast");
}
