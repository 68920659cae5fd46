/*
 * Fortran-ABI drop-in for the m_util_r8 routines an application may call
 * (include/m_util_r8.h:33-66): dmcopy3d_, dmhwr3d_, dmfwr3d_,
 * dminterp3d_, dmdiss3d_ and linbnd3d_ with every argument by pointer, on HOST arrays, as the
 * reference's Fortran takes them. Built as its own library
 * (libpamr_gb300_f77.so) so that an application links it in place of the
 * reference's m_util_r8 object without any source change. Each call copies
 * u1 (and chr1 when excising) and u2 to the device, runs the device
 * routine of libpamr_gb300 (pgb_dm*, pgb_dm*_ex), and copies u2 back; device
 * buffers are kept between calls and grown when needed. The Fortran
 * routines return silently on out-of-range segments; so do these. Errors
 * the Fortran would report with `stop` (unsupported order) are printed and
 * leave u2 unchanged.
 */
#include <cuda_runtime_api.h>
#include <stdio.h>
#include "pamr_gb300.h"

static double *d_buf[5];
static size_t d_cap[5];

static double *dev(int which, const double *h, size_t n)
{
   if (n > d_cap[which]) {
      if (d_buf[which]) cudaFree(d_buf[which]);
      d_buf[which] = 0;
      d_cap[which] = 0;
      if (cudaMalloc((void **)&d_buf[which], n * sizeof(double)) != cudaSuccess) return 0;
      d_cap[which] = n;
   }
   if (h && cudaMemcpy(d_buf[which], h, n * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
      return 0;
   return d_buf[which];
}

static void report(const char *who, int rc)
{
   if (rc) fprintf(stderr, "%s: %s\n", who, pgb_last_error());
}

static int back(double *u2, const double *d2, size_t n)
{
   return cudaMemcpy(u2, d2, n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess;
}

void dmcopy3d_(double *u1, double *u2, int *nx1, int *ny1, int *nz1, int *nx2, int *ny2, int *nz2,
               int *i1, int *j1, int *k1, int *i2, int *j2, int *k2, int *ni, int *nj, int *nk,
               int *si1, int *sj1, int *sk1, int *si2, int *sj2, int *sk2)
{
   size_t n1 = (size_t)*nx1 * *ny1 * *nz1, n2 = (size_t)*nx2 * *ny2 * *nz2;
   double *d1 = dev(0, u1, n1), *d2 = dev(1, u2, n2);
   int rc;
   if (!d1 || !d2) {
      fprintf(stderr, "dmcopy3d: device buffers unavailable\n");
      return;
   }
   rc = pgb_dmcopy3d(d1, d2, *nx1, *ny1, *nz1, *nx2, *ny2, *nz2, *i1, *j1, *k1, *i2, *j2, *k2, *ni,
                     *nj, *nk, *si1, *sj1, *sk1, *si2, *sj2, *sk2, 0);
   if (!rc) rc = back(u2, d2, n2);
   report("dmcopy3d", rc);
}

#define RESTRICT_BODY(name, plain, excised)                                                    \
   size_t n1 = (size_t)*nx1 * *ny1 * *nz1, n2 = (size_t)*nx2 * *ny2 * *nz2;                  \
   double *d1 = dev(0, u1, n1), *d2 = dev(1, u2, n2), *dc = 0;                               \
   int rc;                                                                                   \
   if (*do_ex == 1) dc = dev(2, chr1, n1);                                                   \
   if (!d1 || !d2 || (*do_ex == 1 && !dc)) {                                                 \
      fprintf(stderr, name ": device buffers unavailable\n");                                \
      return;                                                                                \
   }                                                                                         \
   if (*do_ex == 1)                                                                          \
      rc = excised(d1, d2, *nx1, *ny1, *nz1, *nx2, *ny2, *nz2, *i1, *j1, *k1, *i2, *j2, *k2, \
                   *ni, *nj, *nk, *si1, *sj1, *sk1, *si2, *sj2, *sk2, dc, *ex, 0);            \
   else                                                                                      \
      rc = plain(d1, d2, *nx1, *ny1, *nz1, *nx2, *ny2, *nz2, *i1, *j1, *k1, *i2, *j2, *k2,   \
                 *ni, *nj, *nk, *si1, *sj1, *sk1, *si2, *sj2, *sk2, 0);                       \
   if (!rc) rc = back(u2, d2, n2);                                                           \
   report(name, rc);

void dmhwr3d_(double *u1, double *u2, int *nx1, int *ny1, int *nz1, int *nx2, int *ny2, int *nz2,
              int *i1, int *j1, int *k1, int *i2, int *j2, int *k2, int *ni, int *nj, int *nk,
              int *si1, int *sj1, int *sk1, int *si2, int *sj2, int *sk2, double *chr1, double *ex,
              int *do_ex)
{
   /* the Fortran masks the stencil legs by chr1 for any nonzero do_ex but
    * zeroes excised centres only for do_ex = 1 (src/m_util_r8.f:681-715);
    * the device kernels implement do_ex 0 and 1, so other values are refused
    * before anything is written */
   if (*do_ex != 0 && *do_ex != 1) {
      fprintf(stderr, "dmhwr3d: do_ex = %d is not supported (0 or 1); u2 unchanged\n", *do_ex);
      return;
   }
   RESTRICT_BODY("dmhwr3d", pgb_dmhwr3d, pgb_dmhwr3d_ex)
}

void dmfwr3d_(double *u1, double *u2, int *nx1, int *ny1, int *nz1, int *nx2, int *ny2, int *nz2,
              int *i1, int *j1, int *k1, int *i2, int *j2, int *k2, int *ni, int *nj, int *nk,
              int *si1, int *sj1, int *sk1, int *si2, int *sj2, int *sk2, double *chr1, double *ex,
              int *do_ex)
{
   RESTRICT_BODY("dmfwr3d", pgb_dmfwr3d, pgb_dmfwr3d_ex)
}

void dminterp3d_(double *u1, double *u2, int *nx1, int *ny1, int *nz1, int *nx2, int *ny2,
                 int *nz2, int *i1, int *j1, int *k1, int *i2, int *j2, int *k2, int *ni, int *nj,
                 int *nk, int *si1, int *sj1, int *sk1, int *irho, int *jrho, int *krho, int *ord,
                 double *chr1, double *ex, int *do_ex)
{
   size_t n1 = (size_t)*nx1 * *ny1 * *nz1, n2 = (size_t)*nx2 * *ny2 * *nz2;
   double *d1 = dev(0, u1, n1), *d2 = dev(1, u2, n2), *dc = 0;
   int rc;
   if (*do_ex == 1) dc = dev(2, chr1, n1);
   if (!d1 || !d2 || (*do_ex == 1 && !dc)) {
      fprintf(stderr, "dminterp3d: device buffers unavailable\n");
      return;
   }
   if (*do_ex == 1)
      rc = pgb_dminterp3d_ex(d1, d2, *nx1, *ny1, *nz1, *nx2, *ny2, *nz2, *i1, *j1, *k1, *i2, *j2,
                             *k2, *ni, *nj, *nk, *si1, *sj1, *sk1, *irho, *jrho, *krho, *ord, dc,
                             *ex, 0);
   else
      rc = pgb_dminterp3d(d1, d2, *nx1, *ny1, *nz1, *nx2, *ny2, *nz2, *i1, *j1, *k1, *i2, *j2, *k2,
                          *ni, *nj, *nk, *si1, *sj1, *sk1, *irho, *jrho, *krho, *ord, 0);
   if (!rc) rc = back(u2, d2, n2);
   report("dminterp3d", rc);
}

/* Kreiss-Oliger dissipation (src/m_util_r8.f:1690-1956 and its excised
 * variant): f, work, eps (one value, or every point when do_ex < 0), mask
 * and chr (when excising) to the device, pgb_dmdiss3d, f and work back */
void dmdiss3d_(double *f, double *work, double *eps, int *do_bdy, int *phys_bdy_type, int *even, int *odd,
               double *mask, double *mask_off, int *nx, int *ny, int *nz, double *chr, double *ex, int *do_ex)
{
   size_t n = (size_t)*nx * *ny * *nz;
   double *df = dev(0, f, n), *dw = dev(1, 0, n), *de = dev(2, eps, *do_ex < 0 ? n : 1), *dm = dev(3, mask, n);
   double *dc = *do_ex != 0 ? dev(4, chr, n) : 0;
   int rc;
   if (!df || !dw || !de || !dm || (*do_ex != 0 && !dc)) {
      fprintf(stderr, "dmdiss3d: device buffers unavailable\n");
      return;
   }
   rc = pgb_dmdiss3d(df, dw, de, *do_bdy, phys_bdy_type, *even, *odd, dm, *mask_off, *nx, *ny, *nz, dc, *ex,
                     *do_ex, 0);
   if (!rc) rc = back(f, df, n);
   if (!rc) rc = back(work, dw, n);
   report("dmdiss3d", rc);
}

/* linear approach to the boundaries (src/m_util_r8.f:1957-2252): f (and chr
 * when excising) to the device, pgb_linbnd3d, f back */
void linbnd3d_(double *f, int *phys_bdy, int *which_bnd, int *Nx, int *Ny, int *Nz, double *chr, double *ex,
               int *do_ex)
{
   size_t n = (size_t)*Nx * *Ny * *Nz;
   double *df = dev(0, f, n), *dc = 0;
   int rc;
   if (*do_ex != 0) dc = dev(2, chr, n);
   if (!df || (*do_ex != 0 && !dc)) {
      fprintf(stderr, "linbnd3d: device buffers unavailable\n");
      return;
   }
   rc = pgb_linbnd3d(df, phys_bdy, *which_bnd, *Nx, *Ny, *Nz, dc, *ex, *do_ex, 0);
   if (!rc) rc = back(f, df, n);
   report("linbnd3d", rc);
}
