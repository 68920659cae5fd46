/*
 * The reference's own PAMR / AMRD as the drop-in test application's
 * environment: AMRD's init_context reads the parameter file (amrd/io.c:36,
 * variable definitions and MG parameters), PAMR_compose_hierarchy builds
 * the AMR hierarchy (src/pamr.c:259), and u and the two sources are filled
 * on time level 1 of every AMR grid (and the second elliptic variable w in
 * coupled cases). Linked with the reference's C sources
 * (compiled here by tests/dropin/dropin.py from the reference tree, with the
 * oracle's single-rank shims) -- with amrd/mg.c for the golden run.
 *
 * TEST INFRASTRUCTURE: built only where the reference tree exists.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "pamr.h"
#include "amrd.h"
#include "mpi.h"
#include "dropin_case.h"

void init_context(char *pfile);   /* amrd/io.c:36 */

static int same_bbox(const double *a, const double *b, int dim)
{
   int i;
   for (i = 0; i < 2 * dim; i++)
      if (fabs(a[i] - b[i]) > 1e-9 * (1 + fabs(a[i]))) return 0;
   return 1;
}

int env_init(const char *case_path, const char *param_path)
{
   dropin_case c;
   int i, l, nlev = 1, argc = 0;
   char **argv = 0;
   double *bb;
   if (dropin_read_case(case_path, &c)) return 2;
   MPI_Init(&argc, &argv);
   my_rank = 0;
   init_context((char *)param_path);
   bb = (double *)malloc(sizeof(double) * 2 * c.dim * (size_t)c.ngrids);
   for (i = 0; i < c.ngrids; i++) {
      memcpy(&bb[2 * c.dim * i], c.bbox + 6 * i, sizeof(double) * 2 * c.dim);
      if (c.lev[i] > nlev) nlev = c.lev[i];
   }
   if (!PAMR_compose_hierarchy(1, nlev, c.ngrids, c.lev, bb, 0.0)) return 3;
   for (l = 1; l <= nlev; l++) {
      int valid = PAMR_init_s_iter(l, PAMR_AMRH, 0);
      const int gu = PAMR_get_gfn("u", PAMR_AMRH, 1), g0 = PAMR_get_gfn("rho", PAMR_AMRH, 1),
                g1 = PAMR_get_gfn("rho1", PAMR_AMRH, 1), gw_ = c.coupled ? PAMR_get_gfn("w", PAMR_AMRH, 1) : 0;
      while (valid) {
         int rank, dim, gw[6], ngfs, shape[3] = {1, 1, 1};
         double t, *x[3], bbox[6], *gfs[PAMR_MAX_GFNS];
         long n;
         PAMR_get_g_attribs(&rank, &dim, shape, bbox, gw, &t, &ngfs, x, gfs);
         n = (long)shape[0] * shape[1] * shape[2];
         for (i = 0; i < c.ngrids; i++)
            if (c.lev[i] == l && same_bbox(c.bbox + 6 * i, bbox, dim)) break;
         if (i == c.ngrids) return 4;
         memcpy(gfs[gu - 1], c.u[i], sizeof(double) * (size_t)n);
         if (c.coupled) memcpy(gfs[gw_ - 1], c.w[i], sizeof(double) * (size_t)n);
         memcpy(gfs[g0 - 1], c.src0[i], sizeof(double) * (size_t)n);
         memcpy(gfs[g1 - 1], c.src1[i], sizeof(double) * (size_t)n);
         valid = PAMR_next_g();
      }
   }
   return 0;
}
