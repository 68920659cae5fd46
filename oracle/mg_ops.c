/*
 * Per-grid elliptic operators of the CPU checker (see oracle/mg_ops.h).
 *
 * TEST INFRASTRUCTURE (oracle only). Loop nests, 1-based red/black colouring
 * mod(i+j+k+pass,2) and expression order follow examples/nbs/num.f:
 *   lop      num.f:85-123
 *   residual num.f:129-161  (RMS over cmask==ON interior points)
 *   relax    num.f:172-246  (two colour passes; RMS of the in-sweep residual)
 * In 2-D (Nz=1) the k loop is the single plane k=1 and the z terms vanish.
 */
#include <math.h>
#include "mg_ops.h"

#define IDX(g, i, j, k) \
   (((i)-1) + ((j)-1) * (long)(g)->shape[0] + ((k)-1) * (long)(g)->shape[0] * (long)(g)->shape[1])

static const double TWO_PI = 6.283185307179586;   /* 2*pi */
static const double TEN_PI = 31.41592653589793;   /* 5*(2*pi) */

/* lap(u) - as in num.f:113-115, left to right */
static double lap(const oracle_grid *g, const double *v, int i, int j, int k, double dx2,
                  double dy2, double dz2)
{
   double c = v[IDX(g, i, j, k)];
   double t = (v[IDX(g, i + 1, j, k)] - 2 * c + v[IDX(g, i - 1, j, k)]) / dx2 +
              (v[IDX(g, i, j + 1, k)] - 2 * c + v[IDX(g, i, j - 1, k)]) / dy2;
   if (g->dim == 3) t = t + (v[IDX(g, i, j, k + 1)] - 2 * c + v[IDX(g, i, j, k - 1)]) / dz2;
   return t;
}

int oracle_nsrc(int pde) { return pde == ORACLE_NBS || pde == ORACLE_COUPLED ? 2 : 1; }
int oracle_nvar(int pde) { return pde == ORACLE_COUPLED ? 2 : 1; }

/* the source values at point p */
static void src_at(int pde, const double *const *src, long p, double *sv)
{
   int k;
   for (k = 0; k < oracle_nsrc(pde); k++) sv[k] = src[k][p];
}

/* L[u] at one point */
static double op_point(int pde, double t, double u, const double *s)
{
   double p2, p4;
   switch (pde) {
   case ORACLE_CONFORMAL:
      p2 = u * u;
      p4 = p2 * p2;
      return t + TWO_PI * s[0] * (p4 * u);
   case ORACLE_LAPSE:
      return t - s[0] * u;
   case ORACLE_NBS:   /* num.f:113-116: ... - (phi_r(i,j,k)**2+phi_i(i,j,k)**2) */
      return t - (s[0] * s[0] + s[1] * s[1]);
   default:
      return t - s[0];
   }
}

/* dL/du at one point: the Laplacian diagonal j0 plus the source term */
static double jac_point(int pde, double j0, double u, const double *s)
{
   double p2;
   switch (pde) {
   case ORACLE_CONFORMAL:
      p2 = u * u;
      return j0 + TEN_PI * s[0] * (p2 * p2);
   case ORACLE_LAPSE:
      return j0 - s[0];
   default:   /* Poisson, nbs (num.f:236) */
      return j0;
   }
}

static void bounds(const oracle_grid *g, int *ke, int *ks, double *dx2, double *dy2, double *dz2,
                   double *j0)
{
   *dx2 = g->dx[0] * g->dx[0];
   *dy2 = g->dx[1] * g->dx[1];
   if (g->dim == 3) {
      *dz2 = g->dx[2] * g->dx[2];
      *ks = 2;
      *ke = g->shape[2] - 1;
      *j0 = -2 / *dx2 - 2 / *dy2 - 2 / *dz2;
   } else {
      *dz2 = 1;
      *ks = 1;
      *ke = 1;
      *j0 = -2 / *dx2 - 2 / *dy2;
   }
}

void oracle_lop(int pde, const oracle_grid *g, double *lv, const double *v, const double *const *src,
                const double *cmask)
{
   int i, j, k, ks, ke;
   double dx2, dy2, dz2, j0;
   bounds(g, &ke, &ks, &dx2, &dy2, &dz2, &j0);
   for (i = 2; i <= g->shape[0] - 1; i++)
      for (j = 2; j <= g->shape[1] - 1; j++)
         for (k = ks; k <= ke; k++) {
            long p = IDX(g, i, j, k);
            if (cmask[p] == ORACLE_CMASK_ON) {
               double sv[4];
               src_at(pde, src, p, sv);
               lv[p] = op_point(pde, lap(g, v, i, j, k, dx2, dy2, dz2), v[p], sv);
            }
         }
}

double oracle_residual(int pde, const oracle_grid *g, double *res, const double *rhs,
                       const double *v, const double *const *src, const double *cmask)
{
   int i, j, k, ks, ke, sum = 0;
   double dx2, dy2, dz2, j0, norm = 0;
   oracle_lop(pde, g, res, v, src, cmask);
   bounds(g, &ke, &ks, &dx2, &dy2, &dz2, &j0);
   for (i = 2; i <= g->shape[0] - 1; i++)
      for (j = 2; j <= g->shape[1] - 1; j++)
         for (k = ks; k <= ke; k++) {
            long p = IDX(g, i, j, k);
            if (cmask[p] == ORACLE_CMASK_ON) {
               res[p] = res[p] - rhs[p];
               norm = norm + res[p] * res[p];
               sum = sum + 1;
            }
         }
   return sqrt(norm / sum);
}

double oracle_relax(int pde, const oracle_grid *g, double *v, const double *rhs,
                    const double *const *src, const double *cmask)
{
   int i, j, k, ks, ke, pass, sum = 0;
   double dx2, dy2, dz2, j0, norm = 0, res, jac;
   bounds(g, &ke, &ks, &dx2, &dy2, &dz2, &j0);
   for (pass = 0; pass <= 1; pass++)
      for (i = 2; i <= g->shape[0] - 1; i++)
         for (j = 2; j <= g->shape[1] - 1; j++)
            for (k = ks; k <= ke; k++) {
               long p = IDX(g, i, j, k);
               int par = (g->dim == 3) ? (i + j + k + pass) : (i + j + pass);
               if (par % 2 == 0 && cmask[p] == ORACLE_CMASK_ON) {
                  double sv[4];
                  src_at(pde, src, p, sv);
                  res = op_point(pde, lap(g, v, i, j, k, dx2, dy2, dz2), v[p], sv) - rhs[p];
                  jac = jac_point(pde, j0, v[p], sv);
                  v[p] = v[p] - res / jac;
                  norm = norm + res * res;
                  sum = sum + 1;
               }
            }
   return sqrt(norm / sum);
}

/* ------------------------------------------------ two elliptic variables -- */
/* L of variable q of the coupled pair at point p (t its Laplacian) */
static double op_coupled(int q, double t, double u, double w, const double *s)
{
   if (q == 0) return t - s[0] * (u - w) - s[1];
   return t - s[0] * (w - u);
}

void oracle_lop_n(int pde, const oracle_grid *g, double *const *lv, const double *const *v,
                  const double *const *src, const double *cmask)
{
   int i, j, k, ks, ke, q;
   double dx2, dy2, dz2, j0;
   (void)pde;
   bounds(g, &ke, &ks, &dx2, &dy2, &dz2, &j0);
   for (i = 2; i <= g->shape[0] - 1; i++)
      for (j = 2; j <= g->shape[1] - 1; j++)
         for (k = ks; k <= ke; k++) {
            long p = IDX(g, i, j, k);
            if (cmask[p] == ORACLE_CMASK_ON) {
               double sv[4], u = v[0][p], w = v[1][p];
               src_at(ORACLE_COUPLED, src, p, sv);
               for (q = 0; q < 2; q++)
                  lv[q][p] = op_coupled(q, lap(g, v[q], i, j, k, dx2, dy2, dz2), u, w, sv);
            }
         }
}

double oracle_residual_n(int pde, const oracle_grid *g, double *const *res, const double *const *rhs,
                         const double *const *v, const double *const *src, const double *cmask)
{
   int i, j, k, ks, ke, q, sum = 0;
   double dx2, dy2, dz2, j0, norm = 0;
   oracle_lop_n(pde, g, res, v, src, cmask);
   bounds(g, &ke, &ks, &dx2, &dy2, &dz2, &j0);
   for (i = 2; i <= g->shape[0] - 1; i++)
      for (j = 2; j <= g->shape[1] - 1; j++)
         for (k = ks; k <= ke; k++) {
            long p = IDX(g, i, j, k);
            if (cmask[p] == ORACLE_CMASK_ON) {
               for (q = 0; q < 2; q++) {
                  res[q][p] = res[q][p] - rhs[q][p];
                  norm = norm + res[q][p] * res[q][p];
               }
               sum = sum + 1;
            }
         }
   return sqrt(norm / sum);
}

double oracle_relax_n(int pde, const oracle_grid *g, double *const *v, const double *const *rhs,
                      const double *const *src, const double *cmask)
{
   int i, j, k, ks, ke, pass, q, sum = 0;
   double dx2, dy2, dz2, j0, norm = 0, res, jac;
   (void)pde;
   bounds(g, &ke, &ks, &dx2, &dy2, &dz2, &j0);
   for (pass = 0; pass <= 1; pass++)
      for (i = 2; i <= g->shape[0] - 1; i++)
         for (j = 2; j <= g->shape[1] - 1; j++)
            for (k = ks; k <= ke; k++) {
               long p = IDX(g, i, j, k);
               int par = (g->dim == 3) ? (i + j + k + pass) : (i + j + pass);
               if (par % 2 == 0 && cmask[p] == ORACLE_CMASK_ON) {
                  double sv[4];
                  src_at(ORACLE_COUPLED, src, p, sv);
                  for (q = 0; q < 2; q++) {   /* u, then w from the new u */
                     res = op_coupled(q, lap(g, v[q], i, j, k, dx2, dy2, dz2), v[0][p], v[1][p], sv) - rhs[q][p];
                     jac = j0 - sv[0];
                     v[q][p] = v[q][p] - res / jac;
                     norm = norm + res * res;
                  }
                  sum = sum + 1;
               }
            }
   return sqrt(norm / sum);
}
