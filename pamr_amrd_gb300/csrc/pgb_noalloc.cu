/*
 * pgb_residual_norm_noalloc: the residual of one grid and its RMS norm
 * (app_MG_residual's work, examples/nbs/num.f:129-161) computed without
 * allocating any device memory.
 *
 * Who needs it: applications that cannot call cudaMalloc at the point where
 * they want a residual. PAMR-based codes own every grid function themselves
 * (PAMR allocates all grid memory, src/gh.c:1152) and often plan their whole
 * device footprint up front, so a library that grows it on demand breaks
 * their budget; and cudaMalloc/cudaFree can synchronize the device, which a
 * caller issuing asynchronous per-grid work on its own stream cannot allow
 * between launches. The ordinary path (pgb_create / pgb_vcycle) allocates
 * its scratch once per hierarchy; this entry point instead reduces through a
 * fixed array in device global memory that lives for the whole process.
 *
 * Scratch: pgb_noalloc_scratch below, 64 KiB per device that loads the
 * library (held until process exit). It holds one partial sum and one
 * partial count per CTA plus the last-CTA counter, so a grid may need at
 * most PGB_NOALLOC_MAX_TILES CTAs (tiles of 32 x 8 x 8 points); larger grids
 * are rejected with an error before anything is launched.
 *
 * Set-up: host code needs the array's device address, which is not the
 * host-side symbol. The first call on each device (with that device current)
 * looks it up with cudaGetSymbolAddress and caches it; make that first call
 * before any stream capture. Every call shares the one array and leaves its
 * contents behind: each call clears the counter it relies on, but two calls
 * whose kernels overlap on the GPU (e.g. on different streams) race on the
 * scratch and must not be issued that way.
 *
 * Calls no cudaMalloc, cudaFree or allocating library routine.
 */
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>
#include "pamr_gb300.h"

#define NA_TX 32
#define NA_TY 8
#define NA_TZ 8
#define NA_NT (NA_TX * NA_TY)
#define NA_MAX_DEVICES 64

/* per-CTA partial sums [0, MAX), partial counts [MAX, 2*MAX), counter word at 2*MAX */
static __device__ __align__(256) double pgb_noalloc_scratch[2 * PGB_NOALLOC_MAX_TILES + 32];

static void *g_scratch_addr[NA_MAX_DEVICES];
static __thread char g_na_err[256];

/* errors follow PAMR's convention of printing a message (and returning a
 * distinct status code, see pamr_gb300.h) */
static int na_fail(int code)
{
   fprintf(stderr, "%s\n", g_na_err);
   return code;
}

#define TWO_PI 6.283185307179586

__device__ __forceinline__ double na_term(double num, double dx2, double idx2, int pow2)
{
   return pow2 ? num * idx2 : num / dx2;
}

__device__ __forceinline__ double na_sum(double v, double *sm)
{
   int t = threadIdx.x + threadIdx.y * blockDim.x;
   for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
   if ((t & 31) == 0) sm[t >> 5] = v;
   __syncthreads();
   if (t < 32) {
      v = (t < (NA_NT >> 5)) ? sm[t] : 0.0;
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
   }
   __syncthreads();
   return v;
}

struct na_args {
   int pde, dim, n0, n1, n2, pow2, tx, ty, tz;
   double dx2[3], idx2[3];
};

/* one CTA per 32 x 8 x 8 tile, tiles numbered x fastest then y then z */
__global__ void __launch_bounds__(NA_NT) k_residual_noalloc(
   na_args a, const double *u, const double *rhs, const double *src,
   const unsigned char *cmask, double *res, double *norm, double *scratch)
{
   __shared__ double sm[32];
   __shared__ int last;
   const int b = blockIdx.x;
   const int ti = b % a.tx, tj = (b / a.tx) % a.ty, tk = b / (a.tx * a.ty);
   const int i = ti * NA_TX + threadIdx.x, j = tj * NA_TY + threadIdx.y;
   const long sy = a.n0, sz = (long)a.n0 * a.n1;
   double acc = 0, cnt = 0;
   int kz = a.dim == 3 ? NA_TZ : 1;
   for (int kk = 0; kk < kz; kk++) {
      int k = tk * NA_TZ + kk;
      bool in = i >= 1 && i <= a.n0 - 2 && j >= 1 && j <= a.n1 - 2 &&
                (a.dim == 2 ? k == 0 : (k >= 1 && k <= a.n2 - 2));
      if (!in) continue;
      long p = i + sy * j + sz * k;
      if (cmask && !cmask[p]) continue;
      double c = u[p];
      double t = na_term(u[p + 1] - 2 * c + u[p - 1], a.dx2[0], a.idx2[0], a.pow2) +
                 na_term(u[p + sy] - 2 * c + u[p - sy], a.dx2[1], a.idx2[1], a.pow2);
      if (a.dim == 3) t = t + na_term(u[p + sz] - 2 * c + u[p - sz], a.dx2[2], a.idx2[2], a.pow2);
      double s = src[p], l;
      if (a.pde == PGB_PDE_CONFORMAL) {
         double p2 = c * c, p4 = p2 * p2;
         l = t + TWO_PI * s * (p4 * c);
      } else if (a.pde == PGB_PDE_LAPSE)
         l = t - s * c;
      else
         l = t - s;
      double r = l - rhs[p];
      res[p] = r;
      acc += r * r;
      cnt += 1;
   }
   acc = na_sum(acc, sm);
   cnt = na_sum(cnt, sm);
   unsigned int *counter = (unsigned int *)(scratch + 2 * PGB_NOALLOC_MAX_TILES);
   if (threadIdx.x == 0 && threadIdx.y == 0) {
      scratch[b] = acc;
      scratch[PGB_NOALLOC_MAX_TILES + b] = cnt;
   }
   __threadfence();
   __syncthreads();
   if (threadIdx.x == 0 && threadIdx.y == 0) last = (atomicAdd(counter, 1u) == gridDim.x - 1);
   __syncthreads();
   if (!last) return;
   const int t = threadIdx.x + threadIdx.y * blockDim.x;
   double v = 0, c = 0;
   for (int q = t; q < (int)gridDim.x; q += NA_NT) {
      v += __ldcg(&scratch[q]);
      c += __ldcg(&scratch[PGB_NOALLOC_MAX_TILES + q]);
   }
   v = na_sum(v, sm);
   c = na_sum(c, sm);
   if (t == 0) {
      *norm = sqrt(v / c);
      *counter = 0;
   }
}

static void *scratch_address(void)
{
   int dev = 0;
   if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAX_DEVICES) {
      snprintf(g_na_err, sizeof(g_na_err), "pgb_residual_norm_noalloc: no usable current device");
      return 0;
   }
   if (!g_scratch_addr[dev]) {
      void *p = 0;
      cudaError_t e = cudaGetSymbolAddress(&p, pgb_noalloc_scratch);
      if (e != cudaSuccess) {
         snprintf(g_na_err, sizeof(g_na_err), "pgb_residual_norm_noalloc: cudaGetSymbolAddress: %s",
                  cudaGetErrorString(e));
         return 0;
      }
      g_scratch_addr[dev] = p;
   }
   return g_scratch_addr[dev];
}

static int is_pow2(double v)
{
   int e;
   return v > 0 && frexp(v, &e) == 0.5;
}

extern "C" int pgb_residual_norm_noalloc(int pde, int dim, const int *shape3, const double *dx3,
                                         const double *u, const double *rhs, const double *src,
                                         const unsigned char *cmask, double *res, double *norm,
                                         void *stream)
{
   na_args a;
   cudaStream_t st = (cudaStream_t)stream;
   double *scratch;
   long tiles;
   if (pde < 0 || pde > 2 || dim < 2 || dim > 3 || !shape3 || !dx3) {
      snprintf(g_na_err, sizeof(g_na_err), "pgb_residual_norm_noalloc: bad pde, dim or shape");
      return na_fail(1);
   }
   memset(&a, 0, sizeof(a));
   a.pde = pde;
   a.dim = dim;
   a.n0 = shape3[0];
   a.n1 = shape3[1];
   a.n2 = dim == 3 ? shape3[2] : 1;
   if (a.n0 < 3 || a.n1 < 3 || (dim == 3 && a.n2 < 3)) {
      snprintf(g_na_err, sizeof(g_na_err), "pgb_residual_norm_noalloc: grid smaller than 3 points");
      return na_fail(1);
   }
   a.tx = (a.n0 + NA_TX - 1) / NA_TX;
   a.ty = (a.n1 + NA_TY - 1) / NA_TY;
   a.tz = dim == 3 ? (a.n2 + NA_TZ - 1) / NA_TZ : 1;
   tiles = (long)a.tx * a.ty * a.tz;
   if (tiles > PGB_NOALLOC_MAX_TILES) {
      snprintf(g_na_err, sizeof(g_na_err),
               "pgb_residual_norm_noalloc: grid %dx%dx%d needs %ld tiles of 32x8x8 points, "
               "the fixed scratch holds %d",
               a.n0, a.n1, a.n2, tiles, PGB_NOALLOC_MAX_TILES);
      return na_fail(2);
   }
   a.pow2 = 1;
   for (int d = 0; d < 3; d++) {
      double dx = d < dim ? dx3[d] : 1.0;
      a.dx2[d] = dx * dx;
      a.idx2[d] = 1.0 / a.dx2[d];
      if (d < dim && !is_pow2(a.dx2[d])) a.pow2 = 0;
   }
   if (!(scratch = (double *)scratch_address())) return na_fail(3);
   /* the last-CTA counter must start at zero; the partials are rewritten */
   cudaError_t e = cudaMemsetAsync(scratch + 2 * PGB_NOALLOC_MAX_TILES, 0, sizeof(unsigned int), st);
   if (e == cudaSuccess) {
      k_residual_noalloc<<<(unsigned)tiles, dim3(NA_TX, NA_TY), 0, st>>>(a, u, rhs, src, cmask, res,
                                                                          norm, scratch);
      e = cudaGetLastError();
   }
   if (e != cudaSuccess) {
      snprintf(g_na_err, sizeof(g_na_err), "pgb_residual_norm_noalloc: %s", cudaGetErrorString(e));
      return na_fail(4);
   }
   return 0;
}
