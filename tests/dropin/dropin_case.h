/*
 * The case file of the drop-in test application (written by
 * tests/dropin/dropin.py): the AMR hierarchy, the elliptic variable's
 * initial guess and two sources on every grid, the MG parameters, and what
 * the application does (mode 0: solve_elliptics(L, 1, 0); mode 1:
 * PAMR_build_mgh(Lf, Lf, 1) and `arg` vcycle calls with the sources of the
 * finest level changed between them).
 *
 * Layout (little-endian): int32 dim, ngrids, mode, arg, L, coupled, 0, 0;
 * double base_bbox[6]; int32 base_shape[3], 0; int32 ip[10] (pre_swp,
 * pst_swp, max_iter, min_iter, max_citer, min_cwidth, restr_u, restr_res,
 * restr_src, restr_src1); double fp[4] (tol, crtol, w0_r, w0_i); per grid
 * int32 level, shape[3], double bbox[6], then u, [w,] src0, src1 (float64,
 * x fastest). coupled = 1: two elliptic variables u and w (the coupled pair
 * of oracle/mg_ops.h, ORACLE_COUPLED) instead of the nbs potential u.
 */
#ifndef DROPIN_CASE_H
#define DROPIN_CASE_H

#include <stdio.h>
#include <stdlib.h>

typedef struct {
   int dim, ngrids, mode, arg, L, coupled;
   double base_bbox[6];
   int base_shape[3];
   int ip[10];
   double fp[4];
   int *lev, (*shape)[3];
   double *bbox;                    /* 6 per grid */
   double **u, **w, **src0, **src1;   /* w: coupled cases only */
} dropin_case;

static int dropin_read_case(const char *path, dropin_case *c)
{
   FILE *f = fopen(path, "rb");
   int h[8], pad, i;
   if (!f) return 1;
   if (fread(h, 4, 8, f) != 8) goto bad;
   c->dim = h[0];
   c->ngrids = h[1];
   c->mode = h[2];
   c->arg = h[3];
   c->L = h[4];
   c->coupled = h[5];
   if (fread(c->base_bbox, 8, 6, f) != 6 || fread(c->base_shape, 4, 3, f) != 3 || fread(&pad, 4, 1, f) != 1 ||
       fread(c->ip, 4, 10, f) != 10 || fread(c->fp, 8, 4, f) != 4)
      goto bad;
   c->lev = (int *)malloc(sizeof(int) * (size_t)c->ngrids);
   c->shape = (int (*)[3])malloc(sizeof(int) * 3 * (size_t)c->ngrids);
   c->bbox = (double *)calloc(6 * (size_t)c->ngrids, sizeof(double));
   c->u = (double **)malloc(sizeof(double *) * (size_t)c->ngrids);
   c->w = (double **)calloc((size_t)c->ngrids, sizeof(double *));
   c->src0 = (double **)malloc(sizeof(double *) * (size_t)c->ngrids);
   c->src1 = (double **)malloc(sizeof(double *) * (size_t)c->ngrids);
   for (i = 0; i < c->ngrids; i++) {
      long n;
      if (fread(&c->lev[i], 4, 1, f) != 1 || fread(c->shape[i], 4, 3, f) != 3 || fread(c->bbox + 6 * i, 8, 6, f) != 6)
         goto bad;
      n = (long)c->shape[i][0] * c->shape[i][1] * c->shape[i][2];
      c->u[i] = (double *)malloc(sizeof(double) * (size_t)n);
      c->src0[i] = (double *)malloc(sizeof(double) * (size_t)n);
      c->src1[i] = (double *)malloc(sizeof(double) * (size_t)n);
      if (fread(c->u[i], 8, (size_t)n, f) != (size_t)n) goto bad;
      if (c->coupled) {
         c->w[i] = (double *)malloc(sizeof(double) * (size_t)n);
         if (fread(c->w[i], 8, (size_t)n, f) != (size_t)n) goto bad;
      }
      if (fread(c->src0[i], 8, (size_t)n, f) != (size_t)n || fread(c->src1[i], 8, (size_t)n, f) != (size_t)n)
         goto bad;
   }
   fclose(f);
   return 0;
bad:
   fclose(f);
   return 2;
}

#endif
