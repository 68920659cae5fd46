/*
 * Berger-Oliger bookkeeping of the multigrid (elliptic) variables on the
 * device (sm_103a), bit-exact with AMRD's CPU loops (compiled with
 * -fmad=false, same expression order):
 *   extrapolation to the new time level     amrd/evolve.c:344-366
 *   update_mg_extrap_vars                   amrd/evolve.c:1640-1700
 *   set_mg_brs_vars                         amrd/evolve.c:1621-1638
 * The reference loops over AMRD's grid registry; these entry points take
 * the grids of the hierarchy as host arrays of device pointers with their
 * levels, so the elliptic variables and their two extrapolation levels stay
 * on the device across coarse steps. Each grid is one coalesced
 * element-wise launch on the caller's stream.
 */
#include <cuda_runtime.h>
#include <stdio.h>
#include "pgb_dev.h"

static __thread char g_err_bo[256];
static unsigned long long g_launches_bo = 0;

extern "C" unsigned long long pgb_dev_launches_bo(void) { return g_launches_bo; }

static int check_bo(const char *what)
{
   g_launches_bo++;
   cudaError_t e = cudaGetLastError();
   if (e != cudaSuccess) {
      snprintf(g_err_bo, sizeof(g_err_bo), "%s: %s", what, cudaGetErrorString(e));
      pgb_note_error(g_err_bo);
      return 11;
   }
   return 0;
}

static int arg_bo(const char *msg)
{
   snprintf(g_err_bo, sizeof(g_err_bo), "%s", msg);
   pgb_note_error(g_err_bo);
   return 3;
}

static unsigned grid_for(long n)
{
   long b = (n + 255) / 256;
   return (unsigned)(b < 4864 ? (b < 1 ? 1 : b) : 4864);   /* 152 SMs x 32 */
}

/* Element-wise kernels: each thread handles BO_UNROLL elements a block
 * stride apart per iteration, all loads issued before any store, so that
 * enough loads are in flight to stream the arrays at HBM speed. */
#define BO_UNROLL 4

/* mgf0 = f1 etm1 + f2 etm2 (AMRD_MG_EXTRAP_2ND_FROM_ETM1) */
__global__ void k_extrap_etm1(double *mgf0, const double *etm1, const double *etm2, double f1, double f2, long n)
{
   const long step = (long)gridDim.x * blockDim.x;
   for (long j0 = blockIdx.x * (long)blockDim.x + threadIdx.x; j0 < n; j0 += BO_UNROLL * step) {
      double a[BO_UNROLL], b[BO_UNROLL];
#pragma unroll
      for (int u = 0; u < BO_UNROLL; u++) {
         const long j = j0 + u * step;
         a[u] = j < n ? etm1[j] : 0.0;
         b[u] = j < n ? etm2[j] : 0.0;
      }
#pragma unroll
      for (int u = 0; u < BO_UNROLL; u++) {
         const long j = j0 + u * step;
         if (j < n) mgf0[j] = f1 * a[u] + f2 * b[u];
      }
   }
}

/* mgf0 = mgf1 + (dt/dt_lm1) (etm2 - etm1) (AMRD_MG_EXTRAP_2ND_FROM_TN) */
__global__ void k_extrap_tn(double *mgf0, const double *mgf1, const double *etm1, const double *etm2, double ratio,
                            long n)
{
   const long step = (long)gridDim.x * blockDim.x;
   for (long j0 = blockIdx.x * (long)blockDim.x + threadIdx.x; j0 < n; j0 += BO_UNROLL * step) {
      double m[BO_UNROLL], a[BO_UNROLL], b[BO_UNROLL];
#pragma unroll
      for (int u = 0; u < BO_UNROLL; u++) {
         const long j = j0 + u * step;
         m[u] = j < n ? mgf1[j] : 0.0;
         a[u] = j < n ? etm1[j] : 0.0;
         b[u] = j < n ? etm2[j] : 0.0;
      }
#pragma unroll
      for (int u = 0; u < BO_UNROLL; u++) {
         const long j = j0 + u * step;
         if (j < n) mgf0[j] = m[u] + ratio * (b[u] - a[u]);
      }
   }
}

/* etm2 = etm1, etm1 = mgf1, and with correct: etm2 += (etm1 - brs) f */
__global__ void k_extrap_rotate(double *etm1, double *etm2, const double *mgf1, const double *brs, double f,
                                int correct, long n)
{
   const long step = (long)gridDim.x * blockDim.x;
   for (long j0 = blockIdx.x * (long)blockDim.x + threadIdx.x; j0 < n; j0 += BO_UNROLL * step) {
      double e1[BO_UNROLL], m[BO_UNROLL], r[BO_UNROLL];
#pragma unroll
      for (int u = 0; u < BO_UNROLL; u++) {
         const long j = j0 + u * step;
         e1[u] = j < n ? etm1[j] : 0.0;
         m[u] = j < n ? mgf1[j] : 0.0;
         r[u] = (correct && j < n) ? brs[j] : 0.0;
      }
#pragma unroll
      for (int u = 0; u < BO_UNROLL; u++) {
         const long j = j0 + u * step;
         if (j >= n) continue;
         double e2 = e1[u];
         if (correct) e2 += (m[u] - r[u]) * f;
         etm1[j] = m[u];
         etm2[j] = e2;
      }
   }
}

extern "C" int pgb_mg_extrap(int method, double tnp1, double tnp1_lm1, double dt, double dt_lm1, double *mgf0,
                             const double *mgf1, const double *etm1, const double *etm2, long n, void *stream)
{
   if (n < 0 || (method != 0 && method != 1)) return arg_bo("pgb_mg_extrap: bad method or size");
   if (!n) return 0;
   cudaStream_t st = (cudaStream_t)stream;
   if (method == 0) {
      /* the coefficients as evolve.c:350-351 computes them, on the host */
      const double f1 = (tnp1 - (tnp1_lm1 - 2 * dt_lm1)) / dt_lm1;
      const double f2 = -(tnp1 - (tnp1_lm1 - dt_lm1)) / dt_lm1;
      k_extrap_etm1<<<grid_for(n), 256, 0, st>>>(mgf0, etm1, etm2, f1, f2, n);
   } else
      k_extrap_tn<<<grid_for(n), 256, 0, st>>>(mgf0, mgf1, etm1, etm2, dt / dt_lm1, n);
   return check_bo("pgb_mg_extrap");
}

extern "C" int pgb_update_mg_extrap_vars(int L1, int Lf, const int *rho_tm, int ngrids, const int *level,
                                         double *const *etm1, double *const *etm2, const double *const *mgf1,
                                         const double *const *brs, const long *n, double eps_c, void *stream)
{
   cudaStream_t st = (cudaStream_t)stream;
   int lev, g, net_rho;
   if (L1 < 1 || ngrids < 0) return arg_bo("pgb_update_mg_extrap_vars: bad level or grid count");
   /* net_rho as evolve.c:1672-1698 accumulates it: one factor rho_tm[L1-1]
    * (L1 after its increment) per level */
   if (L1 > 1) {
      net_rho = rho_tm[L1 - 1];
      L1++;
   } else
      net_rho = 1;
   for (lev = L1; lev <= Lf; lev++) {
      const int correct = lev > 1 && (eps_c != 0);
      const double f = correct ? 1.0 - eps_c / ((double)net_rho) : 0.0;
      for (g = 0; g < ngrids; g++) {
         if (level[g] != lev || n[g] <= 0) continue;
         k_extrap_rotate<<<grid_for(n[g]), 256, 0, st>>>(etm1[g], etm2[g], mgf1[g], correct ? brs[g] : nullptr, f,
                                                         correct, n[g]);
         if (check_bo("pgb_update_mg_extrap_vars")) return 11;
      }
      net_rho *= rho_tm[L1 - 1];
   }
   return 0;
}

extern "C" int pgb_set_mg_brs_vars(int L1, int L2, int ngrids, const int *level, double *const *brs,
                                   const double *const *mgf1, const long *n, void *stream)
{
   cudaStream_t st = (cudaStream_t)stream;
   for (int lev = L1; lev <= L2; lev++)
      for (int g = 0; g < ngrids; g++) {
         if (level[g] != lev || n[g] <= 0) continue;
         if (cudaMemcpyAsync(brs[g], mgf1[g], sizeof(double) * (size_t)n[g], cudaMemcpyDeviceToDevice, st) !=
             cudaSuccess)
            return check_bo("pgb_set_mg_brs_vars");
      }
   return 0;
}
