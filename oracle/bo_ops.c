/*
 * C restatement of AMRD's Berger-Oliger bookkeeping of the multigrid
 * (elliptic) variables, amrd/evolve.c.
 *
 * TEST INFRASTRUCTURE (oracle only): the checker of libpamr_gb300's device
 * versions (pgb_bo.cu). Each function follows the reference's loop and
 * expression order, so gcc with -ffp-contract=off rounds like it. The
 * reference's functions run on AMRD's global grid registry (PAMR iterators,
 * ev_ldptr); here the grids of the hierarchy are passed as arrays of
 * pointers with their levels. The reference cannot be driven through these
 * functions without its AMRD variable registry, so they are pinned by
 * known-answer tests (tests/test_bo_kat.py), not by running it.
 */
#include "bo_ops.h"

/* extrapolation of the MG variables to the new time level of one grid on a
 * level > 1 (evolve.c:344-366): method 0 (AMRD_MG_EXTRAP_2ND_FROM_ETM1)
 * from the two stored past values, method 1 (AMRD_MG_EXTRAP_2ND_FROM_TN)
 * from the current value and their difference */
int oracle_mg_extrap(int method, double tnp1, double tnp1_lm1, double dt, double dt_lm1, double *mgf0,
                     const double *mgf1, const double *etm1, const double *etm2, long n)
{
   long j;
   double f1 = (tnp1 - (tnp1_lm1 - 2 * dt_lm1)) / dt_lm1;
   double f2 = -(tnp1 - (tnp1_lm1 - dt_lm1)) / dt_lm1;
   if (method == 0) {
      for (j = 0; j < n; j++) mgf0[j] = f1 * etm1[j] + f2 * etm2[j];
   } else if (method == 1) {
      for (j = 0; j < n; j++) mgf0[j] = mgf1[j] + dt / dt_lm1 * (etm2[j] - etm1[j]);
   } else
      return 1;
   return 0;
}

/* update_mg_extrap_vars (evolve.c:1660-1700): on every grid of levels
 * L1..Lf (L1+1..Lf when L1 > 1) extrap_tm1 -> extrap_tm2, the current MG
 * variable -> extrap_tm1, and on levels > 1 with eps_c != 0 the correction
 * extrap_tm2 += (extrap_tm1 - brs) (1 - eps_c / net_rho), net_rho the
 * product of temporal refinement ratios as the reference accumulates it */
void oracle_update_mg_extrap_vars(int L1, int Lf, const int *rho_tm, int ngrids, const int *level, double **etm1,
                                  double **etm2, double *const *mgf1, double *const *brs, const long *n,
                                  double eps_c)
{
   int lev, g, net_rho;
   long j;
   double f;
   if (L1 > 1) {
      net_rho = rho_tm[L1 - 1];
      L1++;
   } else
      net_rho = 1;
   for (lev = L1; lev <= Lf; lev++) {
      for (g = 0; g < ngrids; g++) {
         if (level[g] != lev) continue;
         for (j = 0; j < n[g]; j++) {
            etm2[g][j] = etm1[g][j];
            etm1[g][j] = mgf1[g][j];
         }
         if (lev > 1 && (eps_c != 0)) {
            f = 1.0 - eps_c / ((double)net_rho);
            for (j = 0; j < n[g]; j++) etm2[g][j] += (etm1[g][j] - brs[g][j]) * f;
         }
      }
      net_rho *= rho_tm[L1 - 1];
   }
}

/* set_mg_brs_vars (evolve.c:1624-1638): brs = the current MG variable on
 * every grid of levels L1..L2 */
void oracle_set_mg_brs_vars(int L1, int L2, int ngrids, const int *level, double **brs, double *const *mgf1,
                            const long *n)
{
   int lev, g;
   long j;
   for (lev = L1; lev <= L2; lev++)
      for (g = 0; g < ngrids; g++) {
         if (level[g] != lev) continue;
         for (j = 0; j < n[g]; j++) brs[g][j] = mgf1[g][j];
      }
}
