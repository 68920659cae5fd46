/*
 * C restatement of the grid-function kernels of src/m_util_r8.f that the
 * multigrid path calls (copy, interpolation, half/full-weight restriction).
 *
 * TEST INFRASTRUCTURE (oracle only). The image has no Fortran compiler, so
 * these routines stand in for the reference's Fortran 77 when its C sources
 * are compiled into the CPU checker (oracle/_ref) and are reused by the
 * oracle port (oracle/port). Each routine follows the Fortran line by line:
 * 1-based indices, same loop nests, same left-to-right expression order, so
 * gcc with -ffp-contract=off reproduces the Fortran arithmetic exactly.
 *
 * The excision variants (do_ex=1: dvi2q1d_ex, dvi4q1d_ex, init_chrt,
 * and_chrt, the excised paths of dminterp3d and dmhwr3d, dmfwr3d_ex) are
 * restated too, including two quirks of the Fortran: dmfwr3d_ex's k-only
 * branch adds w3d(i,1,k) (the segment index i, read through the array's
 * column-major storage; an index past its 27 entries, undefined in the
 * Fortran, counts as weight 0 here) and dvi4q1d_ex's right-side
 * extrapolation tests i <= i1s-4*s1. No Fortran compiler is available, so
 * these are pinned by known-answer tests, not by running the reference.
 * dmdiss3d (Kreiss-Oliger dissipation, the evolution kernel next to the
 * elliptic solve) is restated with its excised path (dmdiss3d_ex), and
 * linbnd3d (linear approach to the boundaries) fully. The other
 * evolution-only routines (dmrepop3d1, dmrepop3dc1) are not on the path and
 * abort if reached.
 *
 * Optional call log: when mur8_log_enabled is set, every call records its
 * kernel id and index arguments so a test can compare the reference's
 * transfer bookkeeping with another implementation op by op.
 */
#include <stdio.h>
#include <stdlib.h>
#include "m_util_r8_c.h"

/* ------------------------------------------------------------- call log -- */
int mur8_log_enabled = 0;
mur8_call *mur8_log = 0;
int mur8_log_n = 0, mur8_log_cap = 0;

static void log_call(int kind, const double *u1, const double *u2, const int *iv, int n)
{
   mur8_call *c;
   int i;
   if (!mur8_log_enabled) return;
   if (mur8_log_n == mur8_log_cap) {
      mur8_log_cap = mur8_log_cap ? 2 * mur8_log_cap : 1024;
      mur8_log = (mur8_call *)realloc(mur8_log, sizeof(mur8_call) * (size_t)mur8_log_cap);
   }
   c = &mur8_log[mur8_log_n++];
   c->kind = kind;
   c->u1 = u1;
   c->u2 = u2;
   for (i = 0; i < MUR8_NARGS; i++) c->iv[i] = i < n ? iv[i] : 0;
}

static void not_on_path(const char *who)
{
   fprintf(stderr, "m_util_r8 restatement: %s is not on the multigrid path\n", who);
   abort();
}

/* Fortran u(nx,ny,nz), 1-based (i,j,k) */
#define A3(u, nx, ny, i, j, k) (u)[((i)-1) + ((j)-1) * (long)(nx) + ((k)-1) * (long)(nx) * (long)(ny)]
#define A1(v, i) (v)[(i)-1]

/* src/m_util_r8.f:20-50 */
static void dmcopy3d(const double *u1, double *u2, int nx1, int ny1, int nz1, int nx2, int ny2,
                     int nz2, int i1, int j1, int k1, int i2, int j2, int k2, int ni, int nj, int nk,
                     int si1, int sj1, int sk1, int si2, int sj2, int sk2)
{
   int i, j, k;
   (void)nz2;
   if (i1 < 1 || (i1 + (ni - 1) * si1) > nx1) return;
   if (i2 < 1 || (i2 + (ni - 1) * si2) > nx2) return;
   if (j1 < 1 || (j1 + (nj - 1) * sj1) > ny1) return;
   if (j2 < 1 || (j2 + (nj - 1) * sj2) > ny2) return;
   if (k1 < 1 || (k1 + (nk - 1) * sk1) > nz1) return;
   if (k2 < 1 || (k2 + (nk - 1) * sk2) > nz2) return;
   for (i = 1; i <= ni; i++)
      for (j = 1; j <= nj; j++)
         for (k = 1; k <= nk; k++)
            A3(u2, nx2, ny2, i2 + (i - 1) * si2, j2 + (j - 1) * sj2, k2 + (k - 1) * sk2) =
               A3(u1, nx1, ny1, i1 + (i - 1) * si1, j1 + (j - 1) * sj1, k1 + (k - 1) * sk1);
}

void dmcopy3d_(double *u1, double *u2, int *nx1, int *ny1, int *nz1, int *nx2, int *ny2, int *nz2,
               int *i1, int *j1, int *k1, int *i2, int *j2, int *k2, int *ni, int *nj, int *nk,
               int *si1, int *sj1, int *sk1, int *si2, int *sj2, int *sk2)
{
   int iv[21] = {*nx1, *ny1, *nz1, *nx2, *ny2, *nz2, *i1, *j1, *k1, *i2, *j2, *k2,
                 *ni, *nj, *nk, *si1, *sj1, *sk1, *si2, *sj2, *sk2};
   log_call(MUR8_COPY, u1, u2, iv, 21);
   dmcopy3d(u1, u2, *nx1, *ny1, *nz1, *nx2, *ny2, *nz2, *i1, *j1, *k1, *i2, *j2, *k2, *ni, *nj,
            *nk, *si1, *sj1, *sk1, *si2, *sj2, *sk2);
}

/* src/m_util_r8.f:332-360 (linear, irho:1) */
static void dvi2q1d(const double *v1, double *v2, int i1, int i2, int n1, int n2, int n, int irho,
                    int s1, int s2)
{
   double c0, c1, sg;
   int i, j;
   (void)n1; (void)n2;
   for (i = 1; i <= n; i++) A1(v2, irho * (i - 1) * s2 + i2) = A1(v1, (i - 1) * s1 + i1);
   for (j = 1; j <= irho - 1; j++) {
      sg = (j * 1.0) / irho;
      c0 = 1 - sg;
      c1 = sg;
      for (i = 0; i <= n - 2; i++)
         A1(v2, (irho * i + j) * s2 + i2) = c0 * A1(v1, i * s1 + i1) + c1 * A1(v1, (i + 1) * s1 + i1);
   }
}

/* src/m_util_r8.f:65-144 (cubic, one-sided near the ends, linear if n<4) */
static const double HALF = 0.5, MHALF = -0.5;
static const double SIXTH = 0.16666666666666667, MSIXTH = -0.16666666666666667;

#define CUBIC_COEFS(sg)                                          \
   c0 = MSIXTH * ((sg) - 1.0) * ((sg) - 2.0) * ((sg) - 3.0);     \
   c1 = HALF * (sg) * ((sg) - 2.0) * ((sg) - 3.0);               \
   c2 = MHALF * (sg) * ((sg) - 1.0) * ((sg) - 3.0);              \
   c3 = SIXTH * (sg) * ((sg) - 1.0) * ((sg) - 2.0);

static void dvi4q1d(const double *v1, double *v2, int i1, int i2, int n1, int n2, int n, int irho,
                    int s1, int s2)
{
   double c0, c1, c2, c3, sg;
   int i, j, is, ie;
   if (n < 4) {
      dvi2q1d(v1, v2, i1, i2, n1, n2, n, irho, s1, s2);
      return;
   }
   for (i = 1; i <= n; i++) A1(v2, irho * (i - 1) * s2 + i2) = A1(v1, (i - 1) * s1 + i1);
   if (i1 <= s1) {
      for (j = 1; j <= irho - 1; j++) {
         sg = (j * 1.0) / irho;
         CUBIC_COEFS(sg)
         A1(v2, j * s2 + i2) = c0 * A1(v1, i1) + c1 * A1(v1, s1 + i1) + c2 * A1(v1, 2 * s1 + i1) +
                               c3 * A1(v1, 3 * s1 + i1);
      }
      is = 1;
   } else
      is = 0;
   if ((i1 + n * s1) > (n1 - 2 * s1)) {
      ie = n - 3;
      for (j = 1; j <= irho - 1; j++) {
         sg = 2.0 + (j * 1.0) / irho;
         CUBIC_COEFS(sg)
         A1(v2, (irho * (n - 2) + j) * s2 + i2) =
            c0 * A1(v1, (n - 4) * s1 + i1) + c1 * A1(v1, (n - 3) * s1 + i1) +
            c2 * A1(v1, (n - 2) * s1 + i1) + c3 * A1(v1, (n - 1) * s1 + i1);
      }
   } else
      ie = n - 2;
   for (j = 1; j <= irho - 1; j++) {
      sg = 1.0 + (j * 1.0) / irho;
      CUBIC_COEFS(sg)
      for (i = is; i <= ie; i++)
         A1(v2, (irho * i + j) * s2 + i2) =
            c0 * A1(v1, (i - 1) * s1 + i1) + c1 * A1(v1, i * s1 + i1) +
            c2 * A1(v1, (i + 1) * s1 + i1) + c3 * A1(v1, (i + 2) * s1 + i1);
   }
}

static void dviq1d(int ord, double *v, int i12, int n12, int n, int rho, int s1, int s2)
{
   if (ord == 2) dvi2q1d(v, v, i12, i12, n12, n12, n, rho, s1, s2);
   else dvi4q1d(v, v, i12, i12, n12, n12, n, rho, s1, s2);
}

/* src/m_util_r8.f:368-421: linear interpolation with excision. v1 and v2
 * alias in every call dminterp3d makes; chr1/i3/s3 describe v1's mask on
 * the coarse grid. Writes into the excised zone. */
static void dvi2q1d_ex(double *v1, double *v2, int i1, int i2, int n1, int n2, int n, int irho,
                       int s1, int s2, const double *chr1, int i3, int n3, int s3, double ex)
{
   double c0, c1, sg;
   int i, j, i10, i30;
   (void)n2; (void)n3;
   for (i = 1; i <= n; i++) {
      i10 = (i - 1) * s1 + i1;
      i30 = (i - 1) * s3 + i3;
      if (A1(chr1, i30) == ex) {
         if (i10 > 3 * s1 && A1(chr1, i30 - s3) != ex && A1(chr1, i30 - 2 * s3) != ex &&
             A1(chr1, i30 - 3 * s3) != ex)
            A1(v1, i10) = 3 * (A1(v1, i10 - s1) - A1(v1, i10 - 2 * s1)) + A1(v1, i10 - 3 * s1);
         else if (i10 <= (n1 - 3 * s1) && A1(chr1, i30 + s3) != ex && A1(chr1, i30 + 2 * s3) != ex &&
                  A1(chr1, i30 + 3 * s3) != ex)
            A1(v1, i10) = 3 * (A1(v1, i10 + s1) - A1(v1, i10 + 2 * s1)) + A1(v1, i10 + 3 * s1);
         else if (i10 > 2 * s1 && A1(chr1, i30 - s3) != ex && A1(chr1, i30 - 2 * s3) != ex)
            A1(v1, i10) = 2 * A1(v1, i10 - s1) - A1(v1, i10 - 2 * s1);
         else if (i10 <= (n1 - 2 * s1) && A1(chr1, i30 + s3) != ex && A1(chr1, i30 + 2 * s3) != ex)
            A1(v1, i10) = 2 * A1(v1, i10 + s1) - A1(v1, i10 + 2 * s1);
         else if (i10 > s1 && A1(chr1, i30 - s3) != ex)
            A1(v1, i10) = A1(v1, i10 - s1);
         else if (i10 <= (n1 - s1) && A1(chr1, i30 + s3) != ex)
            A1(v1, i10) = A1(v1, i10 + s1);
      }
      A1(v2, irho * (i - 1) * s2 + i2) = A1(v1, i10);
   }
   for (j = 1; j <= irho - 1; j++) {
      sg = (j * 1.0) / irho;
      c0 = 1 - sg;
      c1 = sg;
      for (i = 0; i <= n - 2; i++) {
         i10 = (irho * i + j) * s2 + i2;
         A1(v2, i10) = c0 * A1(v1, i * s1 + i1) + c1 * A1(v1, (i + 1) * s1 + i1);
      }
   }
}

/* src/m_util_r8.f:153-319: cubic interpolation with excision; falls back
 * to dvi2q1d_ex first when a non-excised run of the (extended) coarse line
 * is shorter than 4, then overwrites with the cubic stencils that apply */
static void dvi4q1d_ex(double *v1, double *v2, int i1, int i2, int n1, int n2, int n, int irho,
                       int s1, int s2, const double *chr1, int i3, int n3, int s3, double ex)
{
   double c0[20], c1[20], c2[20], c3[20], sg;
   int i, j, cn, j0, i1s, i1e, i10, i30, init_2;
   if (irho > 20) {
      fprintf(stderr, "dvi4q1d_ex : irho expected to be less than 20\n");
      abort();
   }
   i = 3;
   i1s = i1;
   while (i > 0 && i1s > s1) {
      i1s = i1s - s1;
      i = i - 1;
   }
   i = 3;
   i1e = i1 + (n - 1) * s1;
   while (i > 0 && i1e < (n1 - s1)) {
      i1e = i1e + s1;
      i = i - 1;
   }
   cn = 0;
   init_2 = 0;
   for (i = i1s; i <= i1e; i += s1) {
      if (A1(chr1, (i - i1) * s3 / s1 + i3) == ex || i == i1e) {
         if (cn > 0 && cn < 4) init_2 = 1;
         else cn = 0;
      } else
         cn = cn + 1;
   }
   if (init_2) dvi2q1d_ex(v1, v2, i1, i2, n1, n2, n, irho, s1, s2, chr1, i3, n3, s3, ex);

#define CH(off) A1(chr1, i3 + s3 * ((off) - i1) / s1)
   for (i = i1s; i <= i1e; i += s1) {
      if (CH(i) == ex) {
         if (i >= (i1s + 3 * s1) && CH(i - s1) != ex && CH(i - 2 * s1) != ex && CH(i - 3 * s1) != ex) {
            if (i >= (i1s + 4 * s1) && CH(i - 4 * s1) != ex)
               A1(v1, i) = 4 * (A1(v1, i - s1) + A1(v1, i - 3 * s1)) - 6 * A1(v1, i - 2 * s1) -
                           A1(v1, i - 4 * s1);
            else
               A1(v1, i) = 3 * (A1(v1, i - s1) - A1(v1, i - 2 * s1)) + A1(v1, i - 3 * s1);
         } else if (i <= (i1e - 3 * s1) && CH(i + s1) != ex && CH(i + 2 * s1) != ex &&
                    CH(i + 3 * s1) != ex) {
            if (i <= (i1s - 4 * s1) && CH(i + 4 * s1) != ex)
               A1(v1, i) = 4 * (A1(v1, i + s1) + A1(v1, i + 3 * s1)) - 6 * A1(v1, i + 2 * s1) -
                           A1(v1, i + 4 * s1);
            else
               A1(v1, i) = 3 * (A1(v1, i + s1) - A1(v1, i + 2 * s1)) + A1(v1, i + 3 * s1);
         }
      }
      if (i >= i1 && i <= (i1 + (n - 1) * s1)) A1(v2, irho * ((i - i1) / s1) * s2 + i2) = A1(v1, i);
   }
#undef CH

   for (j = 1; j <= irho - 1; j++) {   /* left boundary cells */
      sg = (j * 1.0) / irho;
      c0[j - 1] = MSIXTH * (sg - 1.0) * (sg - 2.0) * (sg - 3.0);
      c1[j - 1] = HALF * sg * (sg - 2.0) * (sg - 3.0);
      c2[j - 1] = MHALF * sg * (sg - 1.0) * (sg - 3.0);
      c3[j - 1] = SIXTH * sg * (sg - 1.0) * (sg - 2.0);
   }
   for (i = 1; i <= n - 1; i++) {
      i10 = (i - 1) * s1 + i1;
      i30 = (i - 1) * s3 + i3;
      j0 = (i - 1) * irho * s2 + i2;
      if (i10 <= (i1e - 3 * s1) && A1(chr1, i30 + s3) != ex && A1(chr1, i30 + 2 * s3) != ex &&
          ((i == 1 && i10 == i1s) ||
           (i10 >= (i1s + s1) && A1(chr1, i30) != ex && A1(chr1, i30 - s3) == ex) ||
           A1(chr1, i30) == ex))
         for (j = 1; j <= irho - 1; j++)
            A1(v2, j * s2 + j0) = c0[j - 1] * A1(v1, i10) + c1[j - 1] * A1(v1, s1 + i10) +
                                  c2[j - 1] * A1(v1, 2 * s1 + i10) + c3[j - 1] * A1(v1, 3 * s1 + i10);
   }
   for (j = 1; j <= irho - 1; j++) {   /* right boundary cells */
      sg = 2.0 + (j * 1.0) / irho;
      c0[j - 1] = MSIXTH * (sg - 1.0) * (sg - 2.0) * (sg - 3.0);
      c1[j - 1] = HALF * sg * (sg - 2.0) * (sg - 3.0);
      c2[j - 1] = MHALF * sg * (sg - 1.0) * (sg - 3.0);
      c3[j - 1] = SIXTH * sg * (sg - 1.0) * (sg - 2.0);
   }
   for (i = 1; i <= n - 1; i++) {
      i10 = (i - 1) * s1 + i1;
      i30 = (i - 1) * s3 + i3;
      j0 = (i - 1) * irho * s2 + i2;
      if (i10 >= (i1s + 2 * s1) && A1(chr1, i30 - s3) != ex &&
          ((i == (n - 1) && i10 == (i1e - s1)) ||
           (i10 <= (i1e - s1) && A1(chr1, i30) != ex && A1(chr1, i30 + s3) == ex)))
         for (j = 1; j <= irho - 1; j++)
            A1(v2, j * s2 + j0) = c0[j - 1] * A1(v1, i10 - 2 * s1) + c1[j - 1] * A1(v1, i10 - s1) +
                                  c2[j - 1] * A1(v1, i10) + c3[j - 1] * A1(v1, i10 + s1);
   }
   for (j = 1; j <= irho - 1; j++) {   /* interior */
      sg = 1.0 + (j * 1.0) / irho;
      c0[j - 1] = MSIXTH * (sg - 1.0) * (sg - 2.0) * (sg - 3.0);
      c1[j - 1] = HALF * sg * (sg - 2.0) * (sg - 3.0);
      c2[j - 1] = MHALF * sg * (sg - 1.0) * (sg - 3.0);
      c3[j - 1] = SIXTH * sg * (sg - 1.0) * (sg - 2.0);
   }
   for (i = 1; i <= n; i++) {
      i10 = (i - 1) * s1 + i1;
      i30 = (i - 1) * s3 + i3;
      j0 = (i - 1) * irho * s2 + i2;
      if (A1(chr1, i30) != ex && i10 >= (i1s + s1) && A1(chr1, i30 - s3) != ex &&
          i10 <= (i1e - 2 * s1) && A1(chr1, i30 + s3) != ex)
         for (j = 1; j <= irho - 1; j++)
            A1(v2, j0 + j * s2) = c0[j - 1] * A1(v1, i10 - s1) + c1[j - 1] * A1(v1, i10) +
                                  c2[j - 1] * A1(v1, i10 + s1) + c3[j - 1] * A1(v1, i10 + 2 * s1);
   }
}

/* src/m_util_r8.f:426-456 */
static void init_chrt(double *chrt, const double *chr1, int n, int s3)
{
   int i;
   for (i = 1; i <= n; i++) A1(chrt, i) = A1(chr1, (i - 1) * s3 + 1);
}

static void and_chrt(double *chrt, const double *chr1, int n, int s3, double ex)
{
   int i;
   for (i = 1; i <= n; i++) {
      if (A1(chrt, i) == ex && A1(chr1, (i - 1) * s3 + 1) == ex) A1(chrt, i) = ex;
      else A1(chrt, i) = ex + 1;
   }
}

static void dviq1d_ex(int ord, double *v, int i12, int n12, int n, int rho, int s1, int s2,
                      const double *chr, int i3, int n3, int s3, double ex)
{
   if (ord == 2) dvi2q1d_ex(v, v, i12, i12, n12, n12, n, rho, s1, s2, chr, i3, n3, s3, ex);
   else dvi4q1d_ex(v, v, i12, i12, n12, n12, n, rho, s1, s2, chr, i3, n3, s3, ex);
}

/* src/m_util_r8.f:473-637 */
void dminterp3d_(double *u1, double *u2, int *pnx1, int *pny1, int *pnz1, int *pnx2, int *pny2,
                 int *pnz2, int *pi1, int *pj1, int *pk1, int *pi2, int *pj2, int *pk2, int *pni,
                 int *pnj, int *pnk, int *psi1, int *psj1, int *psk1, int *pirho, int *pjrho,
                 int *pkrho, int *pord, double *chr1, double *ex, int *do_ex)
{
   int nx1 = *pnx1, ny1 = *pny1, nz1 = *pnz1, nx2 = *pnx2, ny2 = *pny2, nz2 = *pnz2;
   int i1 = *pi1, j1 = *pj1, k1 = *pk1, i2 = *pi2, j2 = *pj2, k2 = *pk2;
   int ni = *pni, nj = *pnj, nk = *pnk, si1 = *psi1, sj1 = *psj1, sk1 = *psk1;
   int irho = *pirho, jrho = *pjrho, krho = *pkrho, ord = *pord;
   int i, j, k;
   int iv[24] = {nx1, ny1, nz1, nx2, ny2, nz2, i1, j1, k1, i2, j2, k2,
                 ni, nj, nk, si1, sj1, sk1, irho, jrho, krho, ord, *do_ex, 0};
   log_call(MUR8_INTERP, u1, u2, iv, 24);

   if (i1 < 1 || (i1 + ni - 1) * si1 > nx1) return;
   if (i2 < 1 || (i2 + (ni - 1) * irho) > nx2) return;
   if (j1 < 1 || (j1 + nj - 1) * sj1 > ny1) return;
   if (j2 < 1 || (j2 + (nj - 1) * jrho) > ny2) return;
   if (k1 < 1 || (k1 + nk - 1) * sk1 > nz1) return;
   if (k2 < 1 || (k2 + (nk - 1) * krho) > nz2) return;
   if (!(ord == 2 || ord == 4)) {
      fprintf(stderr, "dminterp3d: only ord=2,4 currently supported\n");
      abort();
   }
   if (*do_ex == 1 && (nx1 > 3000 || ny1 > 3000 || nz1 > 3000)) {
      fprintf(stderr, "dminterp3d: nmax too small\n");
      abort();
   }

   dmcopy3d(u1, u2, nx1, ny1, nz1, nx2, ny2, nz2, i1, j1, k1, i2, j2, k2, ni, nj, nk, si1, sj1,
            sk1, irho, jrho, krho);

   if (*do_ex == 1) {
      double exv = *ex, *chrt = (double *)malloc(sizeof(double) * 3000);
      for (j = j2; j <= j2 + (nj - 1) * jrho; j += jrho)
         for (k = k2; k <= k2 + (nk - 1) * krho; k += krho)
            dviq1d_ex(ord, &A3(u2, nx2, ny2, 1, j, k), i2, nx2, ni, irho, irho, 1,
                      &A3(chr1, nx1, ny1, 1, j1 + sj1 * (j - j2) / jrho, k1 + sk1 * (k - k2) / krho),
                      i1, nx1, si1, exv);
      if (!(nj == 1 && nk == 1)) {
         for (i = i2; i <= i2 + (ni - 1) * irho; i++)
            for (k = k2; k <= k2 + (nk - 1) * krho; k += krho) {
               init_chrt(chrt, &A3(chr1, nx1, ny1, i1 + si1 * ((i - i2) / irho), 1, k1 + sk1 * ((k - k2) / krho)),
                         ny1, nx1);
               if ((i - i2) % irho != 0)
                  and_chrt(chrt, &A3(chr1, nx1, ny1, i1 + si1 * ((i - i2) / irho + 1), 1,
                                     k1 + sk1 * ((k - k2) / krho)), ny1, nx1, exv);
               dviq1d_ex(ord, &A3(u2, nx2, ny2, i, 1, k), 1 + (j2 - 1) * nx2, nx2 * (ny2 - 1) + 1, nj,
                         jrho, jrho * nx2, nx2, chrt, j1, ny1, sj1, exv);
            }
         if (nk != 1)
            for (i = i2; i <= i2 + (ni - 1) * irho; i++)
               for (j = j2; j <= j2 + (nj - 1) * jrho; j++) {
                  init_chrt(chrt, &A3(chr1, nx1, ny1, i1 + si1 * ((i - i2) / irho), j1 + sj1 * ((j - j2) / jrho), 1),
                            nz1, nx1 * ny1);
                  if ((i - i2) % irho != 0)
                     and_chrt(chrt, &A3(chr1, nx1, ny1, i1 + si1 * ((i - i2) / irho + 1),
                                        j1 + sj1 * ((j - j2) / jrho), 1), nz1, nx1 * ny1, exv);
                  if ((j - j2) % jrho != 0)
                     and_chrt(chrt, &A3(chr1, nx1, ny1, i1 + si1 * ((i - i2) / irho),
                                        j1 + sj1 * ((j - j2) / jrho + 1), 1), nz1, nx1 * ny1, exv);
                  if ((j - j2) % jrho != 0 && (i - i2) % irho != 0)
                     and_chrt(chrt, &A3(chr1, nx1, ny1, i1 + si1 * ((i - i2) / irho + 1),
                                        j1 + sj1 * ((j - j2) / jrho + 1), 1), nz1, nx1 * ny1, exv);
                  dviq1d_ex(ord, &A3(u2, nx2, ny2, i, j, 1), (k2 - 1) * nx2 * ny2 + 1,
                            nx2 * ny2 * (nz2 - 1) + 1, nk, krho, krho * nx2 * ny2, nx2 * ny2, chrt,
                            k1, nz1, sk1, exv);
               }
      }
      free(chrt);
      return;
   }

   for (j = j2; j <= j2 + (nj - 1) * jrho; j += jrho)
      for (k = k2; k <= k2 + (nk - 1) * krho; k += krho)
         dviq1d(ord, &A3(u2, nx2, ny2, 1, j, k), i2, nx2, ni, irho, irho, 1);

   if (nj == 1 && nk == 1) return;

   for (i = i2; i <= i2 + (ni - 1) * irho; i++)
      for (k = k2; k <= k2 + (nk - 1) * krho; k += krho)
         dviq1d(ord, &A3(u2, nx2, ny2, i, 1, k), 1 + (j2 - 1) * nx2, nx2 * (ny2 - 1) + 1, nj, jrho,
                jrho * nx2, nx2);

   if (nk == 1) return;

   for (i = i2; i <= i2 + (ni - 1) * irho; i++)
      for (j = j2; j <= j2 + (nj - 1) * jrho; j++)
         dviq1d(ord, &A3(u2, nx2, ny2, i, j, 1), (k2 - 1) * nx2 * ny2 + 1,
                nx2 * ny2 * (nz2 - 1) + 1, nk, krho, krho * nx2 * ny2, nx2 * ny2);
}

/* src/m_util_r8.f:649-723 */
void dmhwr3d_(double *u1, double *u2, int *pnx1, int *pny1, int *pnz1, int *pnx2, int *pny2,
              int *pnz2, int *pi1, int *pj1, int *pk1, int *pi2, int *pj2, int *pk2, int *pni,
              int *pnj, int *pnk, int *psi1, int *psj1, int *psk1, int *psi2, int *psj2,
              int *psk2, double *chr1, double *ex, int *do_ex)
{
   int nx1 = *pnx1, ny1 = *pny1, nz1 = *pnz1, nx2 = *pnx2, ny2 = *pny2, nz2 = *pnz2;
   int i1 = *pi1, j1 = *pj1, k1 = *pk1, i2 = *pi2, j2 = *pj2, k2 = *pk2;
   int ni = *pni, nj = *pnj, nk = *pnk, si1 = *psi1, sj1 = *psj1, sk1 = *psk1;
   int si2 = *psi2, sj2 = *psj2, sk2 = *psk2;
   int i, j, k, w, i0, j0, k0;
   double sum;
   int iv[22] = {nx1, ny1, nz1, nx2, ny2, nz2, i1, j1, k1, i2, j2, k2,
                 ni, nj, nk, si1, sj1, sk1, si2, sj2, sk2, *do_ex};
   log_call(MUR8_HWR, u1, u2, iv, 22);

   if (i1 < 1 || (i1 + (ni - 1) * si1) > nx1) return;
   if (i2 < 1 || (i2 + (ni - 1) * si2) > nx2) return;
   if (j1 < 1 || (j1 + (nj - 1) * sj1) > ny1) return;
   if (j2 < 1 || (j2 + (nj - 1) * sj2) > ny2) return;
   if (k1 < 1 || (k1 + (nk - 1) * sk1) > nz1) return;
   if (k2 < 1 || (k2 + (nk - 1) * sk2) > nz2) return;
#define C3(a, b, c) A3(chr1, nx1, ny1, a, b, c)
   for (i = 1; i <= ni; i++)
      for (j = 1; j <= nj; j++)
         for (k = 1; k <= nk; k++) {
            i0 = i1 + (i - 1) * si1;
            j0 = j1 + (j - 1) * sj1;
            k0 = k1 + (k - 1) * sk1;
            w = 0;
            sum = 0;
            if (i0 > 1 && i0 <= (nx1 - 1)) {
               if (*do_ex == 0 || (C3(i0 - 1, j0, k0) != *ex && C3(i0, j0, k0) != *ex &&
                                   C3(i0 + 1, j0, k0) != *ex)) {
                  w = w + 4;
                  sum = sum + A3(u1, nx1, ny1, i0 - 1, j0, k0) + 2 * A3(u1, nx1, ny1, i0, j0, k0) +
                        A3(u1, nx1, ny1, i0 + 1, j0, k0);
               }
            }
            if (j0 > 1 && j0 <= (ny1 - 1)) {
               if (*do_ex == 0 || (C3(i0, j0 - 1, k0) != *ex && C3(i0, j0, k0) != *ex &&
                                   C3(i0, j0 + 1, k0) != *ex)) {
                  w = w + 4;
                  sum = sum + A3(u1, nx1, ny1, i0, j0 - 1, k0) + 2 * A3(u1, nx1, ny1, i0, j0, k0) +
                        A3(u1, nx1, ny1, i0, j0 + 1, k0);
               }
            }
            if (k0 > 1 && k0 <= (nz1 - 1)) {
               if (*do_ex == 0 || (C3(i0, j0, k0 - 1) != *ex && C3(i0, j0, k0) != *ex &&
                                   C3(i0, j0, k0 + 1) != *ex)) {
                  w = w + 4;
                  sum = sum + A3(u1, nx1, ny1, i0, j0, k0 - 1) + 2 * A3(u1, nx1, ny1, i0, j0, k0) +
                        A3(u1, nx1, ny1, i0, j0, k0 + 1);
               }
            }
            if (*do_ex == 1 && C3(i0, j0, k0) == *ex)
               A3(u2, nx2, ny2, i2 + (i - 1) * si2, j2 + (j - 1) * sj2, k2 + (k - 1) * sk2) = 0;
            else if (w > 0)
               A3(u2, nx2, ny2, i2 + (i - 1) * si2, j2 + (j - 1) * sj2, k2 + (k - 1) * sk2) = sum / w;
            else
               A3(u2, nx2, ny2, i2 + (i - 1) * si2, j2 + (j - 1) * sj2, k2 + (k - 1) * sk2) =
                  A3(u1, nx1, ny1, i0, j0, k0);
         }
#undef C3
}

/* src/m_util_r8.f:835-949, called by dmfwr3d when do_ex=1 (bounds already
 * checked) */
static const int W3D[27] = {1, 2, 1, 2, 4, 2, 1, 2, 1, 2, 4, 2, 4, 8, 4, 2, 4, 2, 1, 2, 1, 2, 4, 2, 1, 2, 1};
/* Fortran w3d(a,b,c) through its column-major storage */
static int w3d(int a, int b, int c)
{
   int o = (a - 1) + 3 * (b - 1) + 9 * (c - 1);
   return o >= 0 && o < 27 ? W3D[o] : 0;
}

static void dmfwr3d_ex(const double *u1, double *u2, int nx1, int ny1, int nz1, int nx2, int ny2,
                       int i1, int j1, int k1, int i2, int j2, int k2, int ni, int nj, int nk,
                       int si1, int sj1, int sk1, int si2, int sj2, int sk2, const double *chr1,
                       double ex)
{
   int i, j, k, i0, j0, k0, im, jm, km, ip, jp, kp, i01, j01, k01, w;
   double sum;
   (void)nz1;
#define U(a, b, c) A3(u1, nx1, ny1, a, b, c)
#define C3(a, b, c) A3(chr1, nx1, ny1, a, b, c)
   for (i = 1; i <= ni; i++)
      for (j = 1; j <= nj; j++)
         for (k = 1; k <= nk; k++) {
            i0 = i1 + (i - 1) * si1;
            j0 = j1 + (j - 1) * sj1;
            k0 = k1 + (k - 1) * sk1;
            im = i0 - 1; jm = j0 - 1; km = k0 - 1;
            ip = i0 + 1; jp = j0 + 1; kp = k0 + 1;
            sum = 0;
            w = 0;
            if (i0 > 1 && i0 <= (nx1 - 1) && j0 > 1 && j0 <= (ny1 - 1) && k0 > 1 && k0 <= (nz1 - 1)) {
               for (i01 = im; i01 <= ip; i01++)
                  for (j01 = jm; j01 <= jp; j01++)
                     for (k01 = km; k01 <= kp; k01++)
                        if (C3(i01, j01, k01) != ex) {
                           sum = sum + w3d(i01 - im + 1, j01 - jm + 1, k01 - km + 1) * U(i01, j01, k01);
                           w = w + w3d(i01 - im + 1, j01 - jm + 1, k01 - km + 1);
                        }
            } else if (i0 > 1 && i0 <= (nx1 - 1) && j0 > 1 && j0 <= (ny1 - 1)) {
               for (i01 = im; i01 <= ip; i01++)
                  for (j01 = jm; j01 <= jp; j01++)
                     if (C3(i01, j01, k0) != ex) {
                        sum = sum + w3d(i01 - im + 1, j01 - jm + 1, 1) * U(i01, j01, k0);
                        w = w + w3d(i01 - im + 1, j01 - jm + 1, 1);
                     }
            } else if (j0 > 1 && j0 <= (ny1 - 1) && k0 > 1 && k0 <= (nz1 - 1)) {
               for (j01 = jm; j01 <= jp; j01++)
                  for (k01 = km; k01 <= kp; k01++)
                     if (C3(i0, j01, k01) != ex) {
                        sum = sum + w3d(1, j01 - jm + 1, k01 - km + 1) * U(i0, j01, k01);
                        w = w + w3d(1, j01 - jm + 1, k01 - km + 1);
                     }
            } else if (i0 > 1 && i0 <= (nx1 - 1) && k0 > 1 && k0 <= (nz1 - 1)) {
               for (i01 = im; i01 <= ip; i01++)
                  for (k01 = km; k01 <= kp; k01++)
                     if (C3(i01, j0, k01) != ex) {
                        sum = sum + w3d(i01 - im + 1, 1, k01 - km + 1) * U(i01, j0, k01);
                        w = w + w3d(i01 - im + 1, 1, k01 - km + 1);
                     }
            } else if (i0 > 1 && i0 <= (nx1 - 1)) {
               for (i01 = im; i01 <= ip; i01++)
                  if (C3(i01, j0, k0) != ex) {
                     sum = sum + w3d(i01 - im + 1, 1, 1) * U(i01, j0, k0);
                     w = w + w3d(i01 - im + 1, 1, 1);
                  }
            } else if (j0 > 1 && j0 <= (ny1 - 1)) {
               for (j01 = jm; j01 <= jp; j01++)
                  if (C3(i0, j01, k0) != ex) {
                     sum = sum + w3d(1, j01 - jm + 1, 1) * U(i0, j01, k0);
                     w = w + w3d(1, j01 - jm + 1, 1);
                  }
            } else if (k0 > 1 && k0 <= (nz1 - 1)) {
               for (k01 = km; k01 <= kp; k01++)
                  if (C3(i0, j0, k01) != ex) {
                     sum = sum + w3d(1, 1, k01 - km + 1) * U(i0, j0, k01);
                     w = w + w3d(i, 1, k01 - km + 1);   /* as written in the Fortran */
                  }
            } else {
               sum = U(i0, j0, k0);
               w = 1;
            }
            if (w == 0 || C3(i0, j0, k0) == ex)
               A3(u2, nx2, ny2, i2 + (i - 1) * si2, j2 + (j - 1) * sj2, k2 + (k - 1) * sk2) = 0;
            else
               A3(u2, nx2, ny2, i2 + (i - 1) * si2, j2 + (j - 1) * sj2, k2 + (k - 1) * sk2) = sum / w;
         }
#undef U
#undef C3
}

/* src/m_util_r8.f:733-830 */
void dmfwr3d_(double *u1, double *u2, int *pnx1, int *pny1, int *pnz1, int *pnx2, int *pny2,
              int *pnz2, int *pi1, int *pj1, int *pk1, int *pi2, int *pj2, int *pk2, int *pni,
              int *pnj, int *pnk, int *psi1, int *psj1, int *psk1, int *psi2, int *psj2,
              int *psk2, double *chr1, double *ex, int *do_ex)
{
   int nx1 = *pnx1, ny1 = *pny1, nz1 = *pnz1, nx2 = *pnx2, ny2 = *pny2, nz2 = *pnz2;
   int i1 = *pi1, j1 = *pj1, k1 = *pk1, i2 = *pi2, j2 = *pj2, k2 = *pk2;
   int ni = *pni, nj = *pnj, nk = *pnk, si1 = *psi1, sj1 = *psj1, sk1 = *psk1;
   int si2 = *psi2, sj2 = *psj2, sk2 = *psk2;
   int i, j, k, i0, j0, k0, im, jm, km, ip, jp, kp;
   double *d;
   int iv[22] = {nx1, ny1, nz1, nx2, ny2, nz2, i1, j1, k1, i2, j2, k2,
                 ni, nj, nk, si1, sj1, sk1, si2, sj2, sk2, *do_ex};
   log_call(MUR8_FWR, u1, u2, iv, 22);

   if (i1 < 1 || (i1 + (ni - 1) * si1) > nx1) return;
   if (i2 < 1 || (i2 + (ni - 1) * si2) > nx2) return;
   if (j1 < 1 || (j1 + (nj - 1) * sj1) > ny1) return;
   if (j2 < 1 || (j2 + (nj - 1) * sj2) > ny2) return;
   if (k1 < 1 || (k1 + (nk - 1) * sk1) > nz1) return;
   if (k2 < 1 || (k2 + (nk - 1) * sk2) > nz2) return;
   if (*do_ex == 1) {
      dmfwr3d_ex(u1, u2, nx1, ny1, nz1, nx2, ny2, i1, j1, k1, i2, j2, k2, ni, nj, nk, si1, sj1, sk1,
                 si2, sj2, sk2, chr1, *ex);
      return;
   }

#define U(a, b, c) A3(u1, nx1, ny1, a, b, c)
   for (i = 1; i <= ni; i++)
      for (j = 1; j <= nj; j++)
         for (k = 1; k <= nk; k++) {
            i0 = i1 + (i - 1) * si1;
            j0 = j1 + (j - 1) * sj1;
            k0 = k1 + (k - 1) * sk1;
            im = i0 - 1; jm = j0 - 1; km = k0 - 1;
            ip = i0 + 1; jp = j0 + 1; kp = k0 + 1;
            d = &A3(u2, nx2, ny2, i2 + (i - 1) * si2, j2 + (j - 1) * sj2, k2 + (k - 1) * sk2);
            if (i0 > 1 && i0 <= (nx1 - 1) && j0 > 1 && j0 <= (ny1 - 1) && k0 > 1 &&
                k0 <= (nz1 - 1)) {
               *d = (U(im, jm, km) + 2 * U(i0, jm, km) + U(ip, jm, km) +
                     2 * U(im, j0, km) + 4 * U(i0, j0, km) + 2 * U(ip, j0, km) +
                     U(im, jp, km) + 2 * U(i0, jp, km) + U(ip, jp, km) +
                     2 * U(im, jm, k0) + 4 * U(i0, jm, k0) + 2 * U(ip, jm, k0) +
                     4 * U(im, j0, k0) + 8 * U(i0, j0, k0) + 4 * U(ip, j0, k0) +
                     2 * U(im, jp, k0) + 4 * U(i0, jp, k0) + 2 * U(ip, jp, k0) +
                     U(im, jm, kp) + 2 * U(i0, jm, kp) + U(ip, jm, kp) +
                     2 * U(im, j0, kp) + 4 * U(i0, j0, kp) + 2 * U(ip, j0, kp) +
                     U(im, jp, kp) + 2 * U(i0, jp, kp) + U(ip, jp, kp)) / 64.0;
            } else if (i0 > 1 && i0 <= (nx1 - 1) && j0 > 1 && j0 <= (ny1 - 1)) {
               *d = (1 * U(im, jm, k0) + 2 * U(i0, jm, k0) + 1 * U(ip, jm, k0) +
                     2 * U(im, j0, k0) + 4 * U(i0, j0, k0) + 2 * U(ip, j0, k0) +
                     1 * U(im, jp, k0) + 2 * U(i0, jp, k0) + 1 * U(ip, jp, k0)) / 16.0;
            } else if (j0 > 1 && j0 <= (ny1 - 1) && k0 > 1 && k0 <= (nz1 - 1)) {
               *d = (1 * U(i0, jm, km) + 2 * U(i0, jm, k0) + 1 * U(i0, jm, kp) +
                     2 * U(i0, j0, km) + 4 * U(i0, j0, k0) + 2 * U(i0, j0, kp) +
                     1 * U(i0, jp, km) + 2 * U(i0, jp, k0) + 1 * U(i0, jp, kp)) / 16.0;
            } else if (i0 > 1 && i0 <= (nx1 - 1) && k0 > 1 && k0 <= (nz1 - 1)) {
               *d = (1 * U(im, j0, km) + 2 * U(im, j0, k0) + 1 * U(im, j0, kp) +
                     2 * U(i0, j0, km) + 4 * U(i0, j0, k0) + 2 * U(i0, j0, kp) +
                     1 * U(ip, j0, km) + 2 * U(ip, j0, k0) + 1 * U(ip, j0, kp)) / 16.0;
            } else if (i0 > 1 && i0 <= (nx1 - 1)) {
               *d = (U(im, j0, k0) + 2 * U(i0, j0, k0) + U(ip, j0, k0)) / 4.0;
            } else if (j0 > 1 && j0 <= (ny1 - 1)) {
               *d = (U(i0, jm, k0) + 2 * U(i0, j0, k0) + U(i0, jp, k0)) / 4.0;
            } else if (k0 > 1 && k0 <= (nz1 - 1)) {
               *d = (U(i0, j0, km) + 2 * U(i0, j0, k0) + U(i0, j0, kp)) / 4.0;
            } else {
               *d = U(i0, j0, k0);
            }
         }
#undef U
}

/* Kreiss-Oliger dissipation term of one point along one dimension
 * (src/m_util_r8.f:1736-1801 for i, 1803-1868 for j, 1870-1935 for k): w
 * points at work(i,j,k), s is the stride of the dimension, p the 1-based
 * position along it and n its extent; lo/hi are the faces' cdo_bdy and
 * phys_bdy_type. Same branches and expression order as the Fortran. */
static double diss_hf(const double *w, long s, int p, int n, int cdo_lo, int cdo_hi, int pbt_lo, int pbt_hi,
                      int even, int odd)
{
   const double w4 = 1.0 / 16.0, w3 = 1.0 / 8.0, w2 = 1.0 / 4.0;
   double f_hf = 0;
#define W(o) w[(o) * s]
   if (p > 2 && p < (n - 1)) {
      f_hf = w4 * (W(-2) + W(2) - 4 * (W(-1) + W(1)) + 6 * W(0));
   } else {
      if (cdo_lo != 0 && n >= 5) {
         if (p == 2 && pbt_lo == odd)
            f_hf = w4 * ((-W(0)) + W(2) - 4 * (W(-1) + W(1)) + 6 * W(0));
         else if (p == 2 && pbt_lo == even)
            f_hf = w4 * ((W(0)) + W(2) - 4 * (W(-1) + W(1)) + 6 * W(0));
         else if (p == 2)
            f_hf = w3 * (-W(-1) + 3 * W(0) - 3 * W(1) + W(2));
         else if (p == 1 && pbt_lo == odd)
            f_hf = w4 * ((-W(2)) + W(2) - 4 * ((-W(1)) + W(1)) + 6 * W(0));
         else if (p == 1 && pbt_lo == even)
            f_hf = w4 * ((W(2)) + W(2) - 4 * ((W(1)) + W(1)) + 6 * W(0));
         else if (p == 1)
            f_hf = w2 * (W(0) - 2 * W(1) + W(2));
      }
      if (cdo_hi != 0 && n >= 5) {
         if (p == (n - 1) && pbt_hi == odd)
            f_hf = w4 * (W(-2) + (-W(0)) - 4 * (W(-1) + W(1)) + 6 * W(0));
         else if (p == (n - 1) && pbt_hi == even)
            f_hf = w4 * (W(-2) + (W(0)) - 4 * (W(-1) + W(1)) + 6 * W(0));
         else if (p == (n - 1))
            f_hf = w3 * (-W(1) + 3 * W(0) - 3 * W(-1) + W(-2));
         else if (p == n && pbt_hi == odd)
            f_hf = w4 * (W(-2) + (-W(-2)) - 4 * (W(-1) + (-W(-1))) + 6 * W(0));
         else if (p == n && pbt_hi == even)
            f_hf = w4 * (W(-2) + (W(-2)) - 4 * (W(-1) + (W(-1))) + 6 * W(0));
         else if (p == n)
            f_hf = w2 * (W(0) - 2 * W(-1) + W(-2));
      }
   }
#undef W
   return f_hf;
}

/* The excised variant's term along one dimension (src/m_util_r8.f:1017-1114
 * for i; the j and k blocks repeat it): the Fortran's thirteen branches in
 * order. X(o): the neighbour at offset o is inside the line and not excised;
 * the Fortran tests chr without range guards, so on short lines it reads
 * outside the array there: a neighbour outside counts as excised here, which
 * skips exactly the branches whose stencil would leave the array. */
static double diss_hf_ex(const double *w, const double *ch, double ex, long s, int p, int n, int pbt_lo,
                         int pbt_hi, int even, int odd, int bo1, int bo2)
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

/* dmdiss3d_ex (src/m_util_r8.f:972-1332) with ind_sweeps = .true.: points
 * whose mask is on and that are not excised; bo1, bo2 from do_bdy (with
 * no_uc_ex_diss = .true., do_bdy = 0 disables the one-sided branches except
 * next to an excised end point); eps(1,1,1) when do_ex > 0, eps(i,j,k) per
 * point when do_ex < 0 */
static void diss_ex(double *f, double *work, const double *eps, int do_bdy, const int *pbt, int even, int odd,
                    const double *mask, double mask_off, int Nx, int Ny, int Nz, const double *chr, double ex,
                    int do_ex)
{
   const long sy = Nx, sz = (long)Nx * Ny, ntot = (long)Nx * Ny * Nz;
   int bo1, bo2, i, j, k, pass, npass, mx = Nx;
   long q;
   if (Ny > mx) mx = Ny;
   if (Nz > mx) mx = Nz;
   if (do_bdy == 0) {
      bo1 = -mx;
      bo2 = bo1;
   } else {
      bo1 = 1;
      bo2 = 2;
   }
   npass = 1;
   if (Ny > 1) npass = 2;
   if (Nz > 1) npass = 3;
   for (pass = 1; pass <= npass; pass++) {
      for (q = 0; q < ntot; q++) work[q] = f[q];
      for (i = 1; i <= Nx; i++)
         for (j = 1; j <= Ny; j++)
            for (k = 1; k <= Nz; k++) {
               const long c = (i - 1) + sy * (j - 1) + sz * (k - 1);
               double f_hf, eps_eff = do_ex < 0 ? eps[c] : eps[0];
               if (!(mask[c] != mask_off && chr[c] != ex)) continue;
               if (pass == 1)
                  f_hf = diss_hf_ex(work + c, chr + c, ex, 1, i, Nx, pbt[0], pbt[1], even, odd, bo1, bo2);
               else if (pass == 2)
                  f_hf = diss_hf_ex(work + c, chr + c, ex, sy, j, Ny, pbt[2], pbt[3], even, odd, bo1, bo2);
               else
                  f_hf = diss_hf_ex(work + c, chr + c, ex, sz, k, Nz, pbt[4], pbt[5], even, odd, bo1, bo2);
               f[c] = f[c] - eps_eff * f_hf;
            }
   }
}

/* dmdiss3d (src/m_util_r8.f:1690-1956), the path without excision:
 * independent sweeps (ind_sweeps = .true.), one pass per dimension of
 * extent > 1 (npass 1, 2 or 3); each pass copies f to work and subtracts
 * eps(1,1,1) times the dissipation term along its dimension at every point
 * whose mask is not mask_off. With do_ex != 0 the Fortran calls
 * dmdiss3d_ex, restated above (diss_ex). */
void dmdiss3d_(double *f, double *work, double *eps, int *do_bdy, int *phys_bdy_type, int *even,
               int *odd, double *mask, double *mask_off, int *nx, int *ny, int *nz, double *chr,
               double *ex, int *do_ex)
{
   const int Nx = *nx, Ny = *ny, Nz = *nz;
   const long sy = Nx, sz = (long)Nx * Ny, ntot = (long)Nx * Ny * Nz;
   int cdo_bdy[6], i, j, k, pass, npass;
   long q;
   double eps_eff;
   if (*do_ex != 0) {
      diss_ex(f, work, eps, *do_bdy, phys_bdy_type, *even, *odd, mask, *mask_off, Nx, Ny, Nz, chr, *ex, *do_ex);
      return;
   }
   for (i = 0; i < 6; i++) {
      cdo_bdy[i] = *do_bdy;
      if (phys_bdy_type[i] == *even || phys_bdy_type[i] == *odd) cdo_bdy[i] = 1;
   }
   eps_eff = eps[0];
   npass = 1;
   if (Ny > 1) npass = 2;
   if (Nz > 1) npass = 3;
   for (pass = 1; pass <= npass; pass++) {
      for (q = 0; q < ntot; q++) work[q] = f[q];
      for (i = 1; i <= Nx; i++)
         for (j = 1; j <= Ny; j++)
            for (k = 1; k <= Nz; k++) {
               const long c = (i - 1) + sy * (j - 1) + sz * (k - 1);
               double f_hf;
               if (mask[c] == *mask_off) continue;
               if (pass == 1)
                  f_hf = diss_hf(work + c, 1, i, Nx, cdo_bdy[0], cdo_bdy[1], phys_bdy_type[0], phys_bdy_type[1],
                                 *even, *odd);
               else if (pass == 2)
                  f_hf = diss_hf(work + c, sy, j, Ny, cdo_bdy[2], cdo_bdy[3], phys_bdy_type[2], phys_bdy_type[3],
                                 *even, *odd);
               else
                  f_hf = diss_hf(work + c, sz, k, Nz, cdo_bdy[4], cdo_bdy[5], phys_bdy_type[4], phys_bdy_type[5],
                                 *even, *odd);
               f[c] = f[c] - eps_eff * f_hf;
            }
   }
}
/* linbnd3d (src/m_util_r8.f:1957-2252): linear approach to the physical
 * (which_bnd 1), AMR (2) or all (3) boundaries: the points one in from a
 * selected face become the mean of their two neighbours across it, edge
 * and corner points of the mean of 4 and 8, in the Fortran's statement
 * order (later statements read what earlier ones wrote). As in the
 * Fortran, the corner conditions read (A .and. B) .or. (all .and. X): the
 * excision test X applies only when all faces are selected. Returns 1 where
 * the Fortran stops (invalid extents; which_bnd outside 1..3, where its pf
 * would be undefined; Ny = 1 with Nz > 1, where it indexes outside f). */
int oracle_linbnd3d(double *f, const int *phys_bdy, int which_bnd, int Nx, int Ny, int Nz, const double *chr,
                    double ex, int do_ex)
{
#define F(i, j, k) f[((i)-1) + (long)Nx * (((j)-1) + (long)Ny * ((k)-1))]
#define X(i, j, k) (chr[((i)-1) + (long)Nx * (((j)-1) + (long)Ny * ((k)-1))] != ex)
#define PB(n) (phys_bdy[(n)-1] == pf || all)
   int i, j, k, pf = -1, all = 0;
   const int ne = do_ex == 0;
   /* the Fortran stops on the first three; with Ny = 1 and Nz > 1 its corner
    * statements index j = Ny-2 < 1, outside f: refused here */
   if (Nx < 3 || Ny == 2 || Nz == 2 || (Ny == 1 && Nz > 1)) return 1;
   if (which_bnd == 3)
      all = 1;   /* the Fortran leaves pf undefined here; -1 matches no face code (0 or 1) */
   else if (which_bnd == 1)
      pf = 1;
   else if (which_bnd == 2)
      pf = 0;
   else
      return 1;
   const int jlo = Ny < 2 ? Ny : 2, jhi = 1 > Ny - 1 ? 1 : Ny - 1;
   const int klo = Nz < 2 ? Nz : 2, khi = 1 > Nz - 1 ? 1 : Nz - 1;

   if (PB(1)) {
      for (j = jlo; j <= jhi; j++)
         for (k = klo; k <= khi; k++)
            if (ne || (X(3, j, k) && X(1, j, k))) F(2, j, k) = 0.5 * (F(3, j, k) + F(1, j, k));
      if (Ny > 1 && PB(3))
         for (k = klo; k <= khi; k++)
            if (ne || (X(3, 3, k) && X(3, 1, k) && X(1, 3, k) && X(1, 1, k)))
               F(2, 2, k) = 0.25 * (F(3, 3, k) + F(1, 3, k) + F(3, 1, k) + F(1, 1, k));
      if (Ny > 1 && PB(4))
         for (k = klo; k <= khi; k++)
            if (ne || (X(3, Ny - 2, k) && X(1, Ny - 2, k) && X(3, Ny, k) && X(1, Ny, k)))
               F(2, Ny - 1, k) = 0.25 * (F(3, Ny - 2, k) + F(1, Ny - 2, k) + F(3, Ny, k) + F(1, Ny, k));
      if (Nz > 1 && PB(5))
         for (j = 2; j <= Ny - 1; j++)
            if (ne || (X(3, j, 3) && X(1, j, 3) && X(3, j, 1) && X(1, j, 1)))
               F(2, j, 2) = 0.25 * (F(3, j, 3) + F(1, j, 3) + F(3, j, 1) + F(1, j, 1));
      if (Nz > 1 && PB(6))
         for (j = 2; j <= Ny - 1; j++)
            if (ne || (X(3, j, Nz - 2) && X(1, j, Nz - 2) && X(3, j, Nz) && X(1, j, Nz)))
               F(2, j, Nz - 1) = 0.25 * (F(3, j, Nz - 2) + F(1, j, Nz - 2) + F(3, j, Nz) + F(1, j, Nz));
      if (Nz > 1 && ((phys_bdy[2] == pf && phys_bdy[4] == pf) ||
                     (all && (ne || (X(3, 3, 3) && X(1, 3, 3) && X(3, 1, 3) && X(3, 3, 1) && X(1, 1, 3) &&
                                     X(1, 3, 1) && X(3, 1, 1) && X(1, 1, 1))))))
         F(2, 2, 2) = 0.125 * (F(3, 3, 3) + F(1, 3, 3) + F(3, 1, 3) + F(3, 3, 1) + F(1, 1, 3) + F(1, 3, 1) +
                               F(3, 1, 1) + F(1, 1, 1));
      if (Nz > 1 && ((phys_bdy[3] == pf && phys_bdy[4] == pf) ||
                     (all && (ne || (X(3, Ny - 2, 3) && X(1, Ny - 2, 3) && X(3, Ny, 3) && X(3, Ny - 2, 1) &&
                                     X(1, Ny, 3) && X(1, Ny - 2, 1) && X(3, Ny, 1) && X(1, Ny, 1))))))
         F(2, Ny - 1, 2) = 0.125 * (F(3, Ny - 2, 3) + F(1, Ny - 2, 3) + F(3, Ny, 3) + F(3, Ny - 2, 1) +
                                    F(1, Ny, 3) + F(1, Ny - 2, 1) + F(3, Ny, 1) + F(1, Ny, 1));
      if (Nz > 1 && ((phys_bdy[2] == pf && phys_bdy[5] == pf) ||
                     (all && (ne || (X(3, 3, Nz - 2) && X(1, 3, Nz - 2) && X(3, 1, Nz - 2) && X(3, 3, Nz) &&
                                     X(1, 1, Nz - 2) && X(1, 3, Nz) && X(3, 1, Nz) && X(1, 1, Nz))))))
         F(2, 2, Nz - 1) = 0.125 * (F(3, 3, Nz - 2) + F(1, 3, Nz - 2) + F(3, 1, Nz - 2) + F(3, 3, Nz) +
                                    F(1, 1, Nz - 2) + F(1, 3, Nz) + F(3, 1, Nz) + F(1, 1, Nz));
      if (Nz > 1 && ((phys_bdy[3] == pf && phys_bdy[5] == pf) ||
                     (all && (ne || (X(3, Ny - 2, Nz - 2) && X(1, Ny - 2, Nz - 2) && X(3, Ny, Nz - 2) &&
                                     X(3, Ny - 2, Nz) && X(1, Ny, Nz - 2) && X(1, Ny - 2, Nz) && X(3, Ny, Nz) &&
                                     X(1, Ny, Nz))))))
         F(2, Ny - 1, Nz - 1) = 0.125 * (F(3, Ny - 2, Nz - 2) + F(1, Ny - 2, Nz - 2) + F(3, Ny, Nz - 2) +
                                         F(3, Ny - 2, Nz) + F(1, Ny, Nz - 2) + F(1, Ny - 2, Nz) + F(3, Ny, Nz) +
                                         F(1, Ny, Nz));
   }

   if (PB(2)) {
      for (j = jlo; j <= jhi; j++)
         for (k = klo; k <= khi; k++)
            if (ne || (X(Nx - 2, j, k) && X(Nx, j, k))) F(Nx - 1, j, k) = 0.5 * (F(Nx - 2, j, k) + F(Nx, j, k));
      if (Ny > 1 && PB(3))
         for (k = klo; k <= khi; k++)
            if (ne || (X(Nx - 2, 3, k) && X(Nx, 3, k) && X(Nx - 2, 1, k) && X(Nx, 1, k)))
               F(Nx - 1, 2, k) = 0.25 * (F(Nx - 2, 3, k) + F(Nx, 3, k) + F(Nx - 2, 1, k) + F(Nx, 1, k));
      if (Ny > 1 && PB(4))
         for (k = klo; k <= khi; k++)
            if (ne || (X(Nx - 2, Ny - 2, k) && X(Nx, Ny - 2, k) && X(Nx - 2, Ny, k) && X(Nx, Ny, k)))
               F(Nx - 1, Ny - 1, k) =
                   0.25 * (F(Nx - 2, Ny - 2, k) + F(Nx, Ny - 2, k) + F(Nx - 2, Ny, k) + F(Nx, Ny, k));
      if (Nz > 1 && PB(5))
         for (j = 2; j <= Ny - 1; j++)
            if (ne || (X(Nx - 2, j, 3) && X(Nx, j, 3) && X(Nx - 2, j, 1) && X(Nx, j, 1)))
               F(Nx - 1, j, 2) = 0.25 * (F(Nx - 2, j, 3) + F(Nx, j, 3) + F(Nx - 2, j, 1) + F(Nx, j, 1));
      if (Nz > 1 && PB(6))
         for (j = 2; j <= Ny - 1; j++)
            if (ne || (X(Nx - 2, j, Nz - 2) && X(Nx, j, Nz - 2) && X(Nx - 2, j, Nz) && X(Nx, j, Nz)))
               F(Nx - 1, j, Nz - 1) =
                   0.25 * (F(Nx - 2, j, Nz - 2) + F(Nx, j, Nz - 2) + F(Nx - 2, j, Nz) + F(Nx, j, Nz));
      if (Nz > 1 && ((phys_bdy[2] == pf && phys_bdy[4] == pf) ||
                     (all && (ne || (X(Nx - 2, 3, 3) && X(Nx, 3, 3) && X(Nx - 2, 1, 3) && X(Nx - 2, 3, 1) &&
                                     X(Nx, 1, 3) && X(Nx, 3, 1) && X(Nx - 2, 1, 1) && X(Nx, 1, 1))))))
         F(Nx - 1, 2, 2) = 0.125 * (F(Nx - 2, 3, 3) + F(Nx, 3, 3) + F(Nx - 2, 1, 3) + F(Nx - 2, 3, 1) +
                                    F(Nx, 1, 3) + F(Nx, 3, 1) + F(Nx - 2, 1, 1) + F(Nx, 1, 1));
      if (Nz > 1 && ((phys_bdy[3] == pf && phys_bdy[4] == pf) ||
                     (all && (ne || (X(Nx - 2, Ny - 2, 3) && X(Nx, Ny - 2, 3) && X(Nx - 2, Ny, 3) &&
                                     X(Nx - 2, Ny - 2, 1) && X(Nx, Ny, 3) && X(Nx, Ny - 2, 1) &&
                                     X(Nx - 2, Ny, 1) && X(Nx, Ny, 1))))))
         F(Nx - 1, Ny - 1, 2) = 0.125 * (F(Nx - 2, Ny - 2, 3) + F(Nx, Ny - 2, 3) + F(Nx - 2, Ny, 3) +
                                         F(Nx - 2, Ny - 2, 1) + F(Nx, Ny, 3) + F(Nx, Ny - 2, 1) +
                                         F(Nx - 2, Ny, 1) + F(Nx, Ny, 1));
      if (Nz > 1 && ((phys_bdy[2] == pf && phys_bdy[5] == pf) ||
                     (all && (ne || (X(Nx - 2, 3, Nz - 2) && X(Nx, 3, Nz - 2) && X(Nx - 2, 1, Nz - 2) &&
                                     X(Nx - 2, 3, Nz) && X(Nx, 1, Nz - 2) && X(Nx, 3, Nz) && X(Nx - 2, 1, Nz) &&
                                     X(Nx, 1, Nz))))))
         F(Nx - 1, 2, Nz - 1) = 0.125 * (F(Nx - 2, 3, Nz - 2) + F(Nx, 3, Nz - 2) + F(Nx - 2, 1, Nz - 2) +
                                         F(Nx - 2, 3, Nz) + F(Nx, 1, Nz - 2) + F(Nx, 3, Nz) + F(Nx - 2, 1, Nz) +
                                         F(Nx, 1, Nz));
      if (Nz > 1 && ((phys_bdy[3] == pf && phys_bdy[5] == pf) ||
                     (all && (ne || (X(Nx - 2, Ny - 2, Nz - 2) && X(Nx, Ny, Nz) && X(Nx, Ny - 2, Nz - 2) &&
                                     X(Nx - 2, Ny, Nz - 2) && X(Nx - 2, Ny - 2, Nz) && X(Nx, Ny, Nz - 2) &&
                                     X(Nx, Ny - 2, Nz) && X(Nx - 2, Ny, Nz))))))
         F(Nx - 1, Ny - 1, Nz - 1) = 0.125 * (F(Nx - 2, Ny - 2, Nz - 2) + F(Nx, Ny, Nz) + F(Nx, Ny - 2, Nz - 2) +
                                              F(Nx - 2, Ny, Nz - 2) + F(Nx - 2, Ny - 2, Nz) + F(Nx, Ny, Nz - 2) +
                                              F(Nx, Ny - 2, Nz) + F(Nx - 2, Ny, Nz));
   }

   if (Ny > 1 && PB(3)) {
      for (i = 3; i <= Nx - 2; i++)
         for (k = klo; k <= khi; k++)
            if (ne || (X(i, 3, k) && X(i, 1, k))) F(i, 2, k) = 0.5 * (F(i, 3, k) + F(i, 1, k));
      if (Nz > 1 && PB(5))
         for (i = 3; i <= Nx - 2; i++)
            if (ne || (X(i, 3, 3) && X(i, 1, 3) && X(i, 3, 1) && X(i, 1, 1)))
               F(i, 2, 2) = 0.25 * (F(i, 3, 3) + F(i, 1, 3) + F(i, 3, 1) + F(i, 1, 1));
      if (Nz > 1 && PB(6))
         for (i = 3; i <= Nx - 2; i++)
            if (ne || (X(i, 3, Nz - 2) && X(i, 1, Nz - 2) && X(i, 3, Nz) && X(i, 1, Nz)))
               F(i, 2, Nz - 1) = 0.25 * (F(i, 3, Nz - 2) + F(i, 1, Nz - 2) + F(i, 3, Nz) + F(i, 1, Nz));
   }

   if (Ny > 1 && PB(4)) {
      for (i = 3; i <= Nx - 2; i++)
         for (k = klo; k <= khi; k++)
            if (ne || (X(i, Ny - 2, k) && X(i, Ny, k))) F(i, Ny - 1, k) = 0.5 * (F(i, Ny - 2, k) + F(i, Ny, k));
      if (Nz > 1 && PB(5))
         for (i = 3; i <= Nx - 2; i++)
            if (ne || (X(i, Ny - 2, 3) && X(i, Ny, 3) && X(i, Ny - 2, 1) && X(i, Ny, 1)))
               F(i, Ny - 1, 2) = 0.25 * (F(i, Ny - 2, 3) + F(i, Ny, 3) + F(i, Ny - 2, 1) + F(i, Ny, 1));
      if (Nz > 1 && PB(6))
         for (i = 3; i <= Nx - 2; i++)
            if (ne || (X(i, Ny - 2, Nz - 2) && X(i, Ny, Nz - 2) && X(i, Ny - 2, Nz) && X(i, Ny, Nz)))
               F(i, Ny - 1, Nz - 1) =
                   0.25 * (F(i, Ny - 2, Nz - 2) + F(i, Ny, Nz - 2) + F(i, Ny - 2, Nz) + F(i, Ny, Nz));
   }

   if (Nz > 1 && PB(5))
      for (i = 3; i <= Nx - 2; i++)
         for (j = 3; j <= Ny - 2; j++)
            if (ne || (X(i, j, 3) && X(i, j, 1))) F(i, j, 2) = 0.5 * (F(i, j, 3) + F(i, j, 1));

   if (Nz > 1 && PB(6))
      for (i = 3; i <= Nx - 2; i++)
         for (j = 3; j <= Ny - 2; j++)
            if (ne || (X(i, j, Nz - 2) && X(i, j, Nz))) F(i, j, Nz - 1) = 0.5 * (F(i, j, Nz - 2) + F(i, j, Nz));
#undef F
#undef X
#undef PB
   return 0;
}

void linbnd3d_(double *f, int *phys_bdy, int *which_bnd, int *Nx, int *Ny, int *Nz, double *chr,
               double *ex, int *do_ex)
{
   if (oracle_linbnd3d(f, phys_bdy, *which_bnd, *Nx, *Ny, *Nz, chr, *ex, *do_ex)) not_on_path("linbnd3d (invalid)");
}
void dmrepop3d1_(double *f, double *chr, double *ex, int *io, int *nx, int *ny, int *nz)
{
   (void)f; (void)chr; (void)ex; (void)io; (void)nx; (void)ny; (void)nz;
   not_on_path("dmrepop3d1");
}
void dmrepop3dc1_(double *chr, double *ex, int *nx, int *ny, int *nz)
{
   (void)chr; (void)ex; (void)nx; (void)ny; (void)nz;
   not_on_path("dmrepop3dc1");
}
