/*
 * Kreiss-Oliger dissipation of libpamr_gb300 (sm_103a): dmdiss3d
 * (src/m_util_r8.f:1690-1956) on device arrays, bit-exact with the Fortran
 * (compiled with -fmad=false; same branches and expression order). The
 * path without excision: one independent pass per dimension of extent > 1;
 * a pass copies f to work (as the Fortran does, so work ends as it does)
 * and then, one thread per point, subtracts eps(1,1,1) times the
 * 4th-difference dissipation term along its dimension where the mask is
 * not mask_off, with the Fortran's one-sided and parity variants at the
 * faces; with do_ex != 0 the excised variant (dmdiss3d_ex,
 * src/m_util_r8.f:972-1332), which also skips excised points and switches
 * to one-sided stencils next to them.
 */
#include <cuda_runtime.h>
#include <stdio.h>
#include "pgb_dev.h"

static __thread char g_err_diss[256];
static unsigned long long g_launches_diss = 0;

extern "C" unsigned long long pgb_dev_launches_diss(void) { return g_launches_diss; }

static int fail_diss(const char *msg, int rc)
{
   snprintf(g_err_diss, sizeof(g_err_diss), "%s", msg);
   pgb_note_error(g_err_diss);
   return rc;
}

static int check_diss(const char *what)
{
   g_launches_diss++;
   cudaError_t e = cudaGetLastError();
   if (e != cudaSuccess) {
      snprintf(g_err_diss, sizeof(g_err_diss), "%s: %s", what, cudaGetErrorString(e));
      pgb_note_error(g_err_diss);
      return 11;
   }
   return 0;
}

struct DissFace {
   int cdo_lo, cdo_hi, pbt_lo, pbt_hi;
};

/* the dissipation term of one point along one dimension (the Fortran's
 * per-dimension block: w at work(i,j,k), stride s, 1-based position p of
 * extent n) */
__device__ __forceinline__ double diss_hf(const double *w, long s, int p, int n, DissFace fc, int even, int odd)
{
   const double w4 = 1.0 / 16.0, w3 = 1.0 / 8.0, w2 = 1.0 / 4.0;
   double f_hf = 0;
#define W(o) w[(o) * s]
   if (p > 2 && p < (n - 1)) {
      f_hf = w4 * (W(-2) + W(2) - 4 * (W(-1) + W(1)) + 6 * W(0));
   } else {
      if (fc.cdo_lo != 0 && n >= 5) {
         if (p == 2 && fc.pbt_lo == odd)
            f_hf = w4 * ((-W(0)) + W(2) - 4 * (W(-1) + W(1)) + 6 * W(0));
         else if (p == 2 && fc.pbt_lo == even)
            f_hf = w4 * ((W(0)) + W(2) - 4 * (W(-1) + W(1)) + 6 * W(0));
         else if (p == 2)
            f_hf = w3 * (-W(-1) + 3 * W(0) - 3 * W(1) + W(2));
         else if (p == 1 && fc.pbt_lo == odd)
            f_hf = w4 * ((-W(2)) + W(2) - 4 * ((-W(1)) + W(1)) + 6 * W(0));
         else if (p == 1 && fc.pbt_lo == even)
            f_hf = w4 * ((W(2)) + W(2) - 4 * ((W(1)) + W(1)) + 6 * W(0));
         else if (p == 1)
            f_hf = w2 * (W(0) - 2 * W(1) + W(2));
      }
      if (fc.cdo_hi != 0 && n >= 5) {
         if (p == (n - 1) && fc.pbt_hi == odd)
            f_hf = w4 * (W(-2) + (-W(0)) - 4 * (W(-1) + W(1)) + 6 * W(0));
         else if (p == (n - 1) && fc.pbt_hi == even)
            f_hf = w4 * (W(-2) + (W(0)) - 4 * (W(-1) + W(1)) + 6 * W(0));
         else if (p == (n - 1))
            f_hf = w3 * (-W(1) + 3 * W(0) - 3 * W(-1) + W(-2));
         else if (p == n && fc.pbt_hi == odd)
            f_hf = w4 * (W(-2) + (-W(-2)) - 4 * (W(-1) + (-W(-1))) + 6 * W(0));
         else if (p == n && fc.pbt_hi == even)
            f_hf = w4 * (W(-2) + (W(-2)) - 4 * (W(-1) + (W(-1))) + 6 * W(0));
         else if (p == n)
            f_hf = w2 * (W(0) - 2 * W(-1) + W(-2));
      }
   }
#undef W
   return f_hf;
}

/* The excised variant's term along one dimension (dmdiss3d_ex,
 * src/m_util_r8.f:1017-1114 and its j, k repeats): the Fortran's thirteen
 * branches in order. X(o): the neighbour at offset o is inside the line
 * and not excised; the Fortran tests chr without range guards and reads
 * outside the array on short lines: a neighbour outside counts as excised
 * here, which skips exactly the branches whose stencil would leave the
 * array (so no access leaves it). */
__device__ __forceinline__ double diss_hf_ex(const double *w, const double *ch, double ex, long s, int p, int n,
                                             int pbt_lo, int pbt_hi, int even, int odd, int bo1, int bo2)
{
   const double w4 = 1.0 / 16.0, w3 = 1.0 / 8.0, w2 = 1.0 / 4.0;
#define W(o) w[(o) * s]
#define X(o) (p + (o) >= 1 && p + (o) <= n && ch[(o) * s] != ex)
   if (p > 2 && p < (n - 1) && X(-2) && X(-1) && X(2) && X(1))
      return w4 * (W(-2) + W(2) - 4 * (W(-1) + W(1)) + 6 * W(0));
   if (p == 2 && pbt_lo == odd && X(-1) && X(2) && X(1))
      return w4 * ((-W(0)) + W(2) - 4 * (W(-1) + W(1)) + 6 * W(0));
   if (p == 1 && pbt_lo == odd && X(2) && X(1))
      return w4 * ((-W(2)) + W(2) - 4 * ((-W(1)) + W(1)) + 6 * W(0));
   if (p == n - 1 && pbt_hi == odd && X(1) && X(-2) && X(-1))
      return w4 * (W(-2) + (-W(0)) - 4 * (W(-1) + W(1)) + 6 * W(0));
   if (p == n && pbt_hi == odd && X(-2) && X(-1))
      return w4 * (W(-2) + (-W(-2)) - 4 * (W(-1) + (-W(-1))) + 6 * W(0));
   if (p == 2 && pbt_lo == even && X(-1) && X(2) && X(1))
      return w4 * ((W(0)) + W(2) - 4 * (W(-1) + W(1)) + 6 * W(0));
   if (p == 1 && pbt_lo == even && X(2) && X(1))
      return w4 * ((W(2)) + W(2) - 4 * ((W(1)) + W(1)) + 6 * W(0));
   if (p == n - 1 && pbt_hi == even && X(1) && X(-2) && X(-1))
      return w4 * (W(-2) + (W(0)) - 4 * (W(-1) + W(1)) + 6 * W(0));
   if (p == n && pbt_hi == even && X(-2) && X(-1))
      return w4 * (W(-2) + (W(-2)) - 4 * (W(-1) + (W(-1))) + 6 * W(0));
   if (p > (2 - bo1) && p < (n - 1) && X(-1) && X(1) && X(2))
      return w3 * (-W(-1) + 3 * W(0) - 3 * W(1) + W(2));
   if (p > 2 && p < (n - 1 + bo1) && X(-1) && X(1) && X(-2))
      return w3 * (-W(1) + 3 * W(0) - 3 * W(-1) + W(-2));
   if ((p > (2 - bo2) || (p == 2 && ch[(1 - p) * s] == ex)) && p < (n - 1) && X(1) && X(2))
      return w2 * (W(0) - 2 * W(1) + W(2));
   if (p > 2 && (p < (n - 1 + bo2) || (p == n - 1 && ch[(n - p) * s] == ex)) && X(-1) && X(-2))
      return w2 * (W(0) - 2 * W(-1) + W(-2));
#undef W
#undef X
   return 0;
}

/* one pass along dimension d of the excised variant: points whose mask is
 * on and that are not excised; eps[0] when do_ex > 0, eps per point when
 * do_ex < 0 */
__global__ void k_diss_ex(double *f, const double *work, const double *eps, const double *mask, double mask_off,
                          const double *chr, double ex, int do_ex, int nx, int ny, int nz, int d, int pbt_lo,
                          int pbt_hi, int even, int odd, int bo1, int bo2)
{
   const int sy = nx, sz = nx * ny, n = sz * nz;   /* below 2^31 points (checked by the caller) */
   for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
      if (!(mask[c] != mask_off && chr[c] != ex)) continue;
      const int k = c / sz, r = c - k * sz, j = r / nx, i = r - j * nx;
      const double eps_eff = do_ex < 0 ? eps[c] : eps[0];
      double f_hf;
      if (d == 0)
         f_hf = diss_hf_ex(work + c, chr + c, ex, 1, i + 1, nx, pbt_lo, pbt_hi, even, odd, bo1, bo2);
      else if (d == 1)
         f_hf = diss_hf_ex(work + c, chr + c, ex, sy, j + 1, ny, pbt_lo, pbt_hi, even, odd, bo1, bo2);
      else
         f_hf = diss_hf_ex(work + c, chr + c, ex, sz, k + 1, nz, pbt_lo, pbt_hi, even, odd, bo1, bo2);
      f[c] = f[c] - eps_eff * f_hf;
   }
}

/* one pass along dimension d (0, 1, 2): f -= eps[0] * term(work) where the
 * mask is on; x fastest, one thread per point */
__global__ void k_diss(double *f, const double *work, const double *eps, const double *mask, double mask_off,
                       int nx, int ny, int nz, int d, DissFace fc, int even, int odd)
{
   const int sy = nx, sz = nx * ny, n = sz * nz;   /* below 2^31 points (checked by the caller) */
   const double eps_eff = eps[0];
   for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
      if (mask[c] == mask_off) continue;
      const int k = c / sz, r = c - k * sz, j = r / nx, i = r - j * nx;
      double f_hf;
      if (d == 0)
         f_hf = diss_hf(work + c, 1, i + 1, nx, fc, even, odd);
      else if (d == 1)
         f_hf = diss_hf(work + c, sy, j + 1, ny, fc, even, odd);
      else
         f_hf = diss_hf(work + c, sz, k + 1, nz, fc, even, odd);
      f[c] = f[c] - eps_eff * f_hf;
   }
}

extern "C" int pgb_dmdiss3d(double *f, double *work, const double *eps, int do_bdy, const int *phys_bdy_type,
                            int even, int odd, const double *mask, double mask_off, int nx, int ny, int nz,
                            const double *chr, double ex, int do_ex, void *stream)
{
   cudaStream_t st = (cudaStream_t)stream;
   if (nx < 1 || ny < 1 || nz < 1) return fail_diss("pgb_dmdiss3d: empty grid", 3);
   if ((long)nx * ny * nz >= (1L << 31)) return fail_diss("pgb_dmdiss3d: grid of 2^31 points or more", 3);
   if (do_ex != 0 && !chr) return fail_diss("pgb_dmdiss3d: do_ex needs chr", 3);
   int cdo[6];
   for (int i = 0; i < 6; i++) {
      cdo[i] = do_bdy;
      if (phys_bdy_type[i] == even || phys_bdy_type[i] == odd) cdo[i] = 1;
   }
   int npass = 1;
   if (ny > 1) npass = 2;
   if (nz > 1) npass = 3;
   const long n = (long)nx * ny * nz;
   const long blocks = (n + 255) / 256;
   const unsigned grid = (unsigned)(blocks < 4864 ? blocks : 4864);
   /* the excised variant's one-sided branches (dmdiss3d_ex): bo1, bo2 from
    * do_bdy, with no_uc_ex_diss = .true. */
   int mx = nx > ny ? nx : ny;
   mx = mx > nz ? mx : nz;
   const int bo1 = do_bdy == 0 ? -mx : 1, bo2 = do_bdy == 0 ? -mx : 2;
   for (int d = 0; d < npass; d++) {
      if (cudaMemcpyAsync(work, f, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
         return check_diss("pgb_dmdiss3d copy");
      if (do_ex != 0)
         k_diss_ex<<<grid, 256, 0, st>>>(f, work, eps, mask, mask_off, chr, ex, do_ex, nx, ny, nz, d,
                                         phys_bdy_type[2 * d], phys_bdy_type[2 * d + 1], even, odd, bo1, bo2);
      else {
         const DissFace fc = {cdo[2 * d], cdo[2 * d + 1], phys_bdy_type[2 * d], phys_bdy_type[2 * d + 1]};
         k_diss<<<grid, 256, 0, st>>>(f, work, eps, mask, mask_off, nx, ny, nz, d, fc, even, odd);
      }
      if (check_diss("pgb_dmdiss3d")) return 11;
   }
   return 0;
}
