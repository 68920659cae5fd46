/*
 * Oracle port (see mg_port.h): the reference's multigrid path restated in
 * plain C for one rank. TEST INFRASTRUCTURE only.
 *
 * Each function names the reference function and file:line it follows.
 * Grid functions on a grid are kept in PAMR's gfn order for this variable
 * set (rho, u, u_res, u_lop, u_rhs, cmask), because local_transfer walks
 * grid functions in that order (src/transfer.c:997).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "mg_port.h"
#include "../mg_ops.h"
#include "../m_util_r8_c.h"

#define MAXLEV 50
#define SMALL_DX 1e-20
#define CMASK_ON 1.0
#define CMASK_OFF 0.0
#define imax(a, b) ((a) > (b) ? (a) : (b))
#define imin(a, b) ((a) < (b) ? (a) : (b))
#define dmax(a, b) (((a) > (b)) ? (a) : (b))
#define dmin(a, b) (((a) < (b)) ? (a) : (b))

enum { G_SRC = 0, G_U, G_RES, G_LOP, G_RHS, G_CMASK, G_SRC1, G_SRC2, G_SRC3, G_W, G_WRES, NGF };
/* G_W, G_WRES: a second elliptic variable and its MG residual, carried (built,
 * injected, synced, interpolated like u and u_res) but never relaxed here:
 * only when port_carry_second_var(1) was called (the drop-in environment's
 * coupled cases, whose solve runs elsewhere) */
static int port_nw = 0;
void port_carry_second_var(int on) { port_nw = on != 0; }
/* source k of the operator (k < oracle_nsrc) */
#define G_SRCK(k) ((k) ? G_SRC1 + (k) - 1 : G_SRC)
static int is_src(int gf) { return gf == G_SRC || gf >= G_SRC1; }
static int src_index(int gf) { return gf == G_SRC ? 0 : gf - G_SRC1 + 1; }

typedef struct pgrid {
   struct pgrid *next;
   int dim, shape[3], coarsest, comm, ghost_width[6];
   double bbox[6];
   double *x[3];
   double *gf[NGF];
   int own[NGF];        /* 1 if this grid allocated gf (else aliased) */
   int own_x;
} pgrid;

typedef struct {
   pgrid *grids;
   double dx[3];
   int in_amrh;
} plev;

typedef struct gsl {
   struct gsl *next;
   double bbox[6];
   pgrid *g;
} gsl;

/* ------------------------------------------------------------ context -- */
static struct {
   const port_case *c;
   int dim;
   double bbox[6];        /* context (base) bbox */
   double amr_dx[MAXLEV][3];
   plev amr[MAXLEV];      /* AMR hierarchy, levels 1..n_amr */
   int n_amr;
   plev mg[MAXLEV];       /* MG hierarchy, levels 1..n_mg */
   int n_mg;
   int tf[NGF];           /* transfer bits of the current communication */
   int frozen;
   int min_level;         /* coarsest AMR level of the MG hierarchy */
   double **sgh_bbox;     /* per AMR level: input bboxes in input order */
   int *sgh_num;
   port_result *r;
} P;

/* variable attributes (amrd/io.c:743-871 for this variable set) */
static int mg_inject_of(int gf)
{
   if (is_src(gf)) {
      const int k = src_index(gf);
      if (k >= oracle_nsrc(P.c->pde)) return 0;   /* a source the operator does not have */
      return k ? P.c->restr_srcx[k - 1] : P.c->restr_src;
   }
   switch (gf) {
   case G_U: return P.c->restr_u;
   case G_RES: return P.c->restr_res;
   case G_W: return port_nw ? P.c->restr_u : 0;
   case G_WRES: return port_nw ? P.c->restr_res : 0;
   default: return 0;
   }
}
static int mg_noinj_to_amr(int gf) { return is_src(gf); }  /* hyperbolic vars */
static int in_amrh(int gf) { return is_src(gf) || gf == G_U || gf == G_CMASK || (port_nw && gf == G_W); }
/* the fields a grid holds: every source the operator reads */
static int used_fields(int mask)
{
   int k;
   for (k = oracle_nsrc(P.c->pde); k < 4; k++) mask &= ~(1 << G_SRCK(k));
   if (!port_nw) mask &= ~((1 << G_W) | (1 << G_WRES));
   return mask;
}

/* misc.c:14-37 */
static int fuzz_eq(double a, double b, double f) { return fabs(b - a) < f; }
static int fuzz_lt(double a, double b, double f) { return a < -f + b; }
static int fuzz_gt(double a, double b, double f) { return a > f + b; }

static long gsize(const pgrid *g) { return (long)g->shape[0] * g->shape[1] * g->shape[2]; }

/* ------------------------------------------------------ transfer bits -- */
/* PAMR_set_tf_bits src/pamr.c:1826-1878 (MGH branch) */
enum { TF_SYNC, TF_INJECT, TF_INJECT_TO_MG_LEV, TF_INTERP, TF_MGH_INIT };
static void set_tf_bits(int stage)
{
   int gf, op;
   if (P.frozen) return;
   for (gf = 0; gf < NGF; gf++) {
      op = 0;
      switch (stage) {
      case TF_SYNC: op = (gf == G_U || (port_nw && gf == G_W)) ? 1 : 0; break;   /* mg_sync = [u (w)] */
      case TF_INJECT: op = mg_noinj_to_amr(gf) ? 0 : mg_inject_of(gf); break;
      case TF_INJECT_TO_MG_LEV: op = mg_inject_of(gf); break;
      case TF_INTERP: op = (gf == G_RES || (port_nw && gf == G_WRES)) ? P.c->interp_order : 0; break;   /* mg_interp2 */
      case TF_MGH_INIT: op = in_amrh(gf) ? mg_inject_of(gf) : 0; break;
      }
      P.tf[gf] = op;
   }
}

/* ------------------------------------------------------ gsl algebra -- */
static gsl *clone_gsl(gsl *p, int first_only)   /* src/transfer.c:40-66 */
{
   gsl *np = 0, *q, *pq = 0;
   while (p) {
      q = (gsl *)malloc(sizeof(gsl));
      if (pq) pq->next = q; else np = q;
      q->next = 0;
      q->g = p->g;
      memcpy(q->bbox, p->bbox, sizeof(q->bbox));
      if (first_only) return np;
      pq = q;
      p = p->next;
   }
   return np;
}

static void free_gsl(gsl *p)
{
   while (p) {
      gsl *q = p;
      p = p->next;
      free(q);
   }
}

static gsl *cat_gsls(gsl *A, gsl *B)   /* src/transfer.c:193-204 */
{
   gsl *cat = A;
   if (!A) return B;
   if (!B) return A;
   while (A->next) A = A->next;
   A->next = B;
   return cat;
}

/* src/transfer.c:73-95 */
static void calc_gs_ibbox(gsl *gs, int *ib, double *dx)
{
   int i;
   pgrid *g = gs->g;
   for (i = 0; i < g->dim; i++) {
      if (g->shape[i] > 1) {
         dx[i] = (g->bbox[2 * i + 1] - g->bbox[2 * i]) / (g->shape[i] - 1);
         ib[2 * i] = (int)((gs->bbox[2 * i] - g->bbox[2 * i]) / dx[i] + 1.01);
         ib[2 * i + 1] = (int)((gs->bbox[2 * i + 1] - g->bbox[2 * i]) / dx[i] + 1.99);
      } else {
         ib[2 * i] = ib[2 * i + 1] = 1;
         dx[i] = SMALL_DX;
      }
   }
}

/* src/transfer.c:101-121 */
static void align_src_bbox(gsl *src, gsl *dst)
{
   int i;
   pgrid *gs = src->g, *gd = dst->g;
   double dxs, dxd;
   for (i = 0; i < gs->dim; i++) {
      if (gs->shape[i] > 1 && gd->shape[i] > 1) {
         dxs = (gs->bbox[2 * i + 1] - gs->bbox[2 * i]) / (gs->shape[i] - 1);
         dxd = (gd->bbox[2 * i + 1] - gd->bbox[2 * i]) / (gd->shape[i] - 1);
         src->bbox[2 * i] = ((int)((src->bbox[2 * i] - gd->bbox[2 * i] + dxs / 2) / dxd)) * dxd +
                            gd->bbox[2 * i];
         if (fuzz_lt(src->bbox[2 * i], gs->bbox[2 * i], dxs / 2)) src->bbox[2 * i] += dxd;
         dst->bbox[2 * i] = src->bbox[2 * i];
         src->bbox[2 * i + 1] =
            ((int)((src->bbox[2 * i + 1] - gd->bbox[2 * i] + dxd - dxs / 2) / dxd)) * dxd +
            gd->bbox[2 * i];
         if (fuzz_gt(src->bbox[2 * i + 1], gs->bbox[2 * i + 1], dxs / 2)) src->bbox[2 * i + 1] -= dxd;
         dst->bbox[2 * i + 1] = src->bbox[2 * i + 1];
      }
   }
}

/* src/transfer.c:132-188 (no ghost zones at one rank, no periodicity) */
static gsl *alloc_gsl(pgrid *g, int interior, int AMR_reduce)
{
   gsl *p = (gsl *)malloc(sizeof(gsl));
   int i, ib[6];
   double dx, dxt[6];
   p->g = g;
   p->next = 0;
   memset(p->bbox, 0, sizeof(p->bbox));
   for (i = 0; i < g->dim; i++) {
      if (g->shape[i] > 1) dx = (g->bbox[2 * i + 1] - g->bbox[2 * i]) / (g->shape[i] - 1);
      else dx = SMALL_DX;
      p->bbox[2 * i] = g->bbox[2 * i];
      p->bbox[2 * i + 1] = g->bbox[2 * i + 1];
      if (interior && g->ghost_width[2 * i])
         p->bbox[2 * i] += g->ghost_width[2 * i] * dx;
      else if (AMR_reduce > 0 && !g->ghost_width[2 * i]) {
         if (fuzz_gt(p->bbox[2 * i], P.bbox[2 * i], dx / 2)) p->bbox[2 * i] += AMR_reduce * dx;
      }
      if (interior && g->ghost_width[2 * i + 1])
         p->bbox[2 * i + 1] += -g->ghost_width[2 * i + 1] * dx;
      else if (AMR_reduce > 0 && !g->ghost_width[2 * i + 1]) {
         if (fuzz_lt(p->bbox[2 * i + 1], P.bbox[2 * i + 1], dx / 2))
            p->bbox[2 * i + 1] += -AMR_reduce * dx;
      }
      if (interior || AMR_reduce) {
         calc_gs_ibbox(p, ib, dxt);
         if ((ib[2 * i + 1] - ib[2 * i] + 1) < 1) {
            free(p);
            return 0;
         }
      }
   }
   return p;
}

/* src/transfer.c:218-285 */
static gsl *gs_subtract(gsl *A, gsl *B)
{
   double cut[6], dx[3];
   int d = A->g->dim, i, j;
   gsl *C = 0, *q;
   if (!B) return clone_gsl(A, 1);
   for (i = 0; i < d; i++) {
      cut[2 * i] = A->bbox[2 * i];
      cut[2 * i + 1] = A->bbox[2 * i + 1];
      if (A->g->shape[i] > 1) dx[i] = (A->g->bbox[2 * i + 1] - A->g->bbox[2 * i]) / (A->g->shape[i] - 1);
      else dx[i] = SMALL_DX;
      if (fuzz_gt(B->bbox[2 * i], A->bbox[2 * i + 1], dx[i] / 2) ||
          fuzz_gt(A->bbox[2 * i], B->bbox[2 * i + 1], dx[i] / 2))
         return clone_gsl(A, 1);
   }
   for (i = 0; i < d; i++) {
      cut[2 * i] = dmax(A->bbox[2 * i], B->bbox[2 * i]);
      if (fuzz_gt(cut[2 * i], A->bbox[2 * i], dx[i] / 2)) {
         q = clone_gsl(A, 1);
         if (C) q->next = C;
         C = q;
         for (j = 0; j < d; j++) {
            if (i == j) {
               C->bbox[2 * i] = A->bbox[2 * i];
               C->bbox[2 * i + 1] = dmax(C->bbox[2 * i], cut[2 * i] - dx[i]);
            } else {
               C->bbox[2 * j] = cut[2 * j];
               C->bbox[2 * j + 1] = cut[2 * j + 1];
            }
         }
      }
      cut[2 * i + 1] = dmin(A->bbox[2 * i + 1], B->bbox[2 * i + 1]);
      if (fuzz_lt(cut[2 * i + 1], A->bbox[2 * i + 1], dx[i] / 2)) {
         q = clone_gsl(A, 1);
         if (C) q->next = C;
         C = q;
         for (j = 0; j < d; j++) {
            if (i == j) {
               C->bbox[2 * i + 1] = A->bbox[2 * i + 1];
               C->bbox[2 * i] = dmin(C->bbox[2 * i + 1], cut[2 * i + 1] + dx[i]);
            } else {
               C->bbox[2 * j] = cut[2 * j];
               C->bbox[2 * j + 1] = cut[2 * j + 1];
            }
         }
      }
   }
   return C;
}

/* src/transfer.c:287-314 */
static gsl *gsl_subtract(gsl *A, gsl *B)
{
   gsl *C = clone_gsl(A, 0), *C0, *C1;
   while (B) {
      C0 = 0;
      C1 = C;
      while (C1) {
         C0 = cat_gsls(C0, gs_subtract(C1, B));
         C1 = C1->next;
      }
      free_gsl(C);
      C = C0;
      B = B->next;
   }
   return C;
}

/* src/transfer.c:325-356 */
static int gs_and(gsl *A, gsl *B, gsl **A0, gsl **B0)
{
   double nb[6], dxA, dxB, dxm;
   int d = A->g->dim, i;
   *A0 = *B0 = 0;
   for (i = 0; i < d; i++) {
      dxA = A->g->shape[i] > 1 ? (A->g->bbox[2 * i + 1] - A->g->bbox[2 * i]) / (A->g->shape[i] - 1) : SMALL_DX;
      dxB = B->g->shape[i] > 1 ? (B->g->bbox[2 * i + 1] - B->g->bbox[2 * i]) / (B->g->shape[i] - 1) : SMALL_DX;
      dxm = dmax(dxA, dxB);
      nb[2 * i] = dmax(A->bbox[2 * i], B->bbox[2 * i]);
      nb[2 * i + 1] = dmin(A->bbox[2 * i + 1], B->bbox[2 * i + 1]);
      if (fuzz_lt(nb[2 * i + 1], nb[2 * i], dxm / 2)) return 0;
   }
   *A0 = clone_gsl(A, 1);
   *B0 = clone_gsl(B, 1);
   for (i = 0; i < d; i++) {
      (*A0)->bbox[2 * i] = (*B0)->bbox[2 * i] = nb[2 * i];
      (*A0)->bbox[2 * i + 1] = (*B0)->bbox[2 * i + 1] = nb[2 * i + 1];
   }
   return 1;
}

/* src/transfer.c:364-386 */
static void extend_gsl(gsl *gs)
{
   int i;
   double dx;
   while (gs) {
      pgrid *g = gs->g;
      for (i = 0; i < g->dim; i++)
         if (g->shape[i] > 1) {
            dx = (g->bbox[2 * i + 1] - g->bbox[2 * i]) / (g->shape[i] - 1);
            gs->bbox[2 * i] = dmax(gs->bbox[2 * i] - dx, g->bbox[2 * i]);
            gs->bbox[2 * i + 1] = dmin(gs->bbox[2 * i + 1] + dx, g->bbox[2 * i + 1]);
         }
      gs = gs->next;
   }
}

/* src/transfer.c:415-458 */
static gsl *build_owned_gsl(plev *lev, int interior, int extend)
{
   gsl *owned = 0, *int_gs, *int_gsl = 0;
   int cint = interior ? 1 : 0, cred = interior > 1 ? interior - 1 : 0;
   pgrid *g;
   for (g = lev->grids; g; g = g->next) {
      if (!g->comm) continue;
      int_gs = alloc_gsl(g, cint, cred);
      owned = cat_gsls(owned, gsl_subtract(int_gs, int_gsl));
      int_gsl = cat_gsls(int_gsl, int_gs);
   }
   if (extend && owned) extend_gsl(owned);
   free_gsl(int_gsl);
   return owned;
}

/* src/transfer.c:465-504 (AMR_bdy_only = 0) */
static gsl *build_complete_gsl(plev *lev)
{
   gsl *c = 0;
   pgrid *g;
   for (g = lev->grids; g; g = g->next)
      if (g->comm) c = cat_gsls(c, alloc_gsl(g, 0, 0));
   return c;
}

/* src/transfer.c:514-540 */
static void build_gstl(gsl *in_src, gsl *in_dst, gsl **os, gsl **od)
{
   gsl *d, *s, *d2;
   *os = *od = 0;
   for (; in_src; in_src = in_src->next)
      for (d = in_dst; d; d = d->next) {
         if (in_src->g == d->g) continue;
         if (gs_and(in_src, d, &s, &d2)) {
            *os = cat_gsls(*os, s);
            *od = cat_gsls(*od, d2);
         }
      }
}

/* src/transfer.c:545-575 */
static int calc_delta(gsl *src, gsl *dst, int *irho)
{
   double dxsm = 0, dxdm = 0;
   int i;
   *irho = 0;
   for (i = 0; i < src->g->dim; i++)
      if (src->g->shape[i] > 1 && dst->g->shape[i] > 1) {
         dxsm = dmax(dxsm, (src->g->bbox[2 * i + 1] - src->g->bbox[2 * i]) / (src->g->shape[i] - 1));
         dxdm = dmax(dxdm, (dst->g->bbox[2 * i + 1] - dst->g->bbox[2 * i]) / (dst->g->shape[i] - 1));
      }
   if (dxsm == 0 || dxdm == 0) return 0;
   if (fuzz_eq(dxsm, dxdm, dxsm / 100)) return 0;
   if (fuzz_gt(dxsm, dxdm, dxsm / 100)) {
      *irho = (int)(dxsm / dxdm + 0.5);
      return -1;
   }
   *irho = (int)(dxdm / dxsm + 0.5);
   return 1;
}

/* src/transfer.c:946-1163 (one rank, no excision) */
static void local_transfer(gsl *src, gsl *dst)
{
   int dim = P.dim, i, one = 1, delta, irho, ib[6], ibd[6];
   int nx1, ny1, nz1, nx2, ny2, nz2, i1, j1, k1, i2, j2, k2, ni, nj, nk;
   int nib, njb, nkb, nx1b, ny1b, nz1b, i2b, j2b, k2b;
   int i1i, i2i, nii, j1i, j2i, nji, k1i, k2i, nki;
   int zero = 0, ord;
   double dx[6], dxd[6], ex = 0, *data;
   int ib_buf = P.c->interp_buffer;
   pgrid *g1, *g2;
   for (; src && dst; src = src->next, dst = dst->next) {
      delta = calc_delta(src, dst, &irho);
      if (delta == 1) align_src_bbox(src, dst);
      calc_gs_ibbox(src, ib, dx);
      calc_gs_ibbox(dst, ibd, dxd);
      g1 = src->g;
      g2 = dst->g;
      for (i = 0; i < NGF; i++) {
         if (!P.tf[i]) continue;
         ni = nj = nk = i1 = i2 = j1 = j2 = k1 = k2 = nx1 = ny1 = nz1 = nx2 = ny2 = nz2 = 1;
         nib = njb = nkb = nx1b = ny1b = nz1b = i2b = j2b = k2b = 1;
         nii = nji = nki = i1i = j1i = k1i = i2i = j2i = k2i = 1;
         if (dim >= 3) {
            k1 = ib[4]; k2 = ibd[4]; nk = ib[5] - ib[4] + 1;
            nz1 = g1->shape[2]; nz2 = g2->shape[2]; nkb = ibd[5] - ibd[4] + 1;
            if (delta == -1) {
               k2b = (int)((src->bbox[4] - g1->bbox[4]) / dxd[2] + 1.5);
               k2i = imax(1, (((k2b - 1) / irho) - ib_buf) * irho + 1);
               k1i = (k2i - 1) / irho + 1;
               nki = imin(nz1, (k2b + nkb - 1) / irho + 1 + ib_buf + 1) - k1i + 1;
               nz1b = (nki - 1) * irho + 1;
               k2b = k2b - k2i + 1;
            }
         }
         if (dim >= 2) {
            j1 = ib[2]; j2 = ibd[2]; nj = ib[3] - ib[2] + 1;
            ny1 = g1->shape[1]; ny2 = g2->shape[1]; njb = ibd[3] - ibd[2] + 1;
            if (delta == -1) {
               j2b = (int)((src->bbox[2] - g1->bbox[2]) / dxd[1] + 1.5);
               j2i = imax(1, (((j2b - 1) / irho) - ib_buf) * irho + 1);
               j1i = (j2i - 1) / irho + 1;
               nji = imin(ny1, (j2b + njb - 1) / irho + 1 + ib_buf + 1) - j1i + 1;
               ny1b = (nji - 1) * irho + 1;
               j2b = j2b - j2i + 1;
            }
         }
         i1 = ib[0]; i2 = ibd[0]; ni = ib[1] - ib[0] + 1;
         nx1 = g1->shape[0]; nx2 = g2->shape[0]; nib = ibd[1] - ibd[0] + 1;
         if (delta == -1) {
            i2b = (int)((src->bbox[0] - g1->bbox[0]) / dxd[0] + 1.5);
            i2i = imax(1, (((i2b - 1) / irho) - ib_buf) * irho + 1);
            i1i = (i2i - 1) / irho + 1;
            nii = imin(nx1, (i2b + nib - 1) / irho + 1 + ib_buf + 1) - i1i + 1;
            nx1b = (nii - 1) * irho + 1;
            i2b = i2b - i2i + 1;
         }
         if (delta == 0) {
            dmcopy3d_(g1->gf[i], g2->gf[i], &nx1, &ny1, &nz1, &nx2, &ny2, &nz2, &i1, &j1, &k1, &i2,
                      &j2, &k2, &ni, &nj, &nk, &one, &one, &one, &one, &one, &one);
         } else if (delta == -1) {
            ord = P.tf[i];
            data = (double *)malloc(sizeof(double) * (size_t)nx1b * ny1b * nz1b);
            dminterp3d_(g1->gf[i], data, &nx1, &ny1, &nz1, &nx1b, &ny1b, &nz1b, &i1i, &j1i, &k1i,
                        &one, &one, &one, &nii, &nji, &nki, &one, &one, &one, &irho, &irho, &irho,
                        &ord, g1->gf[i], &ex, &zero);
            dmcopy3d_(data, g2->gf[i], &nx1b, &ny1b, &nz1b, &nx2, &ny2, &nz2, &i2b, &j2b, &k2b,
                      &i2, &j2, &k2, &nib, &njb, &nkb, &one, &one, &one, &one, &one, &one);
            free(data);
         } else if (delta == 1) {
            if (P.tf[i] == 1)
               dmcopy3d_(g1->gf[i], g2->gf[i], &nx1, &ny1, &nz1, &nx2, &ny2, &nz2, &i1, &j1, &k1,
                         &i2, &j2, &k2, &nib, &njb, &nkb, &irho, &irho, &irho, &one, &one, &one);
            else if (P.tf[i] == 2)
               dmhwr3d_(g1->gf[i], g2->gf[i], &nx1, &ny1, &nz1, &nx2, &ny2, &nz2, &i1, &j1, &k1,
                        &i2, &j2, &k2, &nib, &njb, &nkb, &irho, &irho, &irho, &one, &one, &one,
                        g1->gf[i], &ex, &zero);
            else if (P.tf[i] == 3)
               dmfwr3d_(g1->gf[i], g2->gf[i], &nx1, &ny1, &nz1, &nx2, &ny2, &nz2, &i1, &j1, &k1,
                        &i2, &j2, &k2, &nib, &njb, &nkb, &irho, &irho, &irho, &one, &one, &one,
                        g1->gf[i], &ex, &zero);
         }
      }
   }
}

/* src/pamr.c:533-593 (one rank) */
static void communicate(plev *l1, plev *l2, int interior, int extend)
{
   gsl *src, *dst, *ts, *td;
   src = build_owned_gsl(l1, interior, extend);
   dst = build_complete_gsl(l2);
   if (dst) {
      build_gstl(src, dst, &ts, &td);
      local_transfer(ts, td);
      free_gsl(ts);
      free_gsl(td);
   }
   free_gsl(dst);
   free_gsl(src);
}

static void pamr_sync(int L, int AMR_bdy_width)   /* src/pamr.c:601-617 */
{
   set_tf_bits(TF_SYNC);
   communicate(&P.mg[L], &P.mg[L], 1 + AMR_bdy_width, 0);
}

static void pamr_interp(int Lc)                     /* src/pamr.c:623-638 */
{
   set_tf_bits(TF_INTERP);
   communicate(&P.mg[Lc], &P.mg[Lc + 1], 0, 1);
}

static void pamr_inject(int Lf)                     /* src/pamr.c:667-685 */
{
   if (!P.mg[Lf - 1].in_amrh) set_tf_bits(TF_INJECT_TO_MG_LEV);
   else set_tf_bits(TF_INJECT);
   communicate(&P.mg[Lf], &P.mg[Lf - 1], 1, 0);
}

/* ----------------------------------------------- hierarchy construction -- */
/* src/gh.c:235-257 */
static void insert_grid(plev *lev, pgrid *g)
{
   pgrid *cg = lev->grids, *pg = 0;
   int dim = g->dim;
   while (cg && (cg->bbox[0] < g->bbox[0]) && ((dim < 2) || cg->bbox[2] < g->bbox[2]) &&
          ((dim < 3) || cg->bbox[4] < g->bbox[4]) && (cg->bbox[1] < g->bbox[1]) &&
          ((dim < 2) || cg->bbox[3] < g->bbox[3]) && ((dim < 3) || cg->bbox[5] < g->bbox[5])) {
      pg = cg;
      cg = cg->next;
   }
   g->next = cg;
   if (pg) pg->next = g; else lev->grids = g;
}

/* a grid as compose_cgh makes it at one rank (src/gh.c:696-905): bbox upper
 * edges recomputed from the level spacing, x by accumulation */
static pgrid *new_grid(const double *bbox, const double *lev_dx)
{
   pgrid *g = (pgrid *)calloc(1, sizeof(pgrid));
   int d, m;
   double x, dx;
   g->dim = P.dim;
   g->comm = 1;
   g->shape[0] = g->shape[1] = g->shape[2] = 1;
   for (d = 0; d < P.dim; d++) {
      int n = (int)((bbox[2 * d + 1] - bbox[2 * d]) / lev_dx[d] + 1.5);   /* build_sgh gh.c:352 */
      g->shape[d] = n;
      g->bbox[2 * d] = bbox[2 * d] + lev_dx[d] * 0;
      g->bbox[2 * d + 1] = bbox[2 * d] + lev_dx[d] * (n - 1);
   }
   for (d = 0; d < P.dim; d++) {
      g->x[d] = (double *)malloc(sizeof(double) * (size_t)g->shape[d]);
      dx = (g->bbox[2 * d + 1] - g->bbox[2 * d]) / (g->shape[d] - 1);
      for (m = 0, x = g->bbox[2 * d]; m < g->shape[d]; m++, x += dx) g->x[d][m] = x;
   }
   g->own_x = 1;
   return g;
}

static void alloc_fields(pgrid *g, int which_mask)
{
   int h;
   for (h = 0; h < NGF; h++)
      if ((which_mask >> h) & 1) {
         g->gf[h] = (double *)calloc((size_t)gsize(g), sizeof(double));
         g->own[h] = 1;
      }
}

/* calc_island_no src/gh.c:1427-1467 */
static void calc_island_no(const double *bb, int num, double *island, const double *dx, int cf)
{
   int i, j, k, delta = 1, shape, overlap;
   int mcw = P.c->min_cwidth;
   for (i = 0; i < num; i++) {
      island[i] = i + 1;
      for (j = 0; j < P.dim; j++) {
         shape = (int)((bb[2 * i * P.dim + 2 * j + 1] - bb[2 * i * P.dim + 2 * j]) / dx[j] + 1.5);
         if ((((shape - 1) % cf) && ((shape - 1) / cf + 1) >= mcw) || (((shape - 1) / cf + 1) < mcw))
            island[i] = 0;
         else if (((shape - 1) / cf / 2 + 1) < mcw)
            island[i] = -fabs(island[i]);
      }
   }
   while (delta) {
      delta = 0;
      for (i = 0; i < num; i++)
         for (j = i + 1; j < num; j++)
            if (island[i] != island[j]) {
               overlap = 1;
               for (k = 0; k < P.dim; k++)
                  if (fuzz_gt(bb[2 * i * P.dim + 2 * k], bb[2 * j * P.dim + 2 * k + 1], dx[k] / 2) ||
                      fuzz_gt(bb[2 * i * P.dim + 2 * k + 1], bb[2 * j * P.dim + 2 * k], dx[k] / 2))
                     overlap = 0;
               if (overlap) {
                  delta++;
                  if (island[i] == 0 || island[j] == 0) island[i] = island[j] = 0;
                  else island[i] = island[j] = dmin(island[i], island[j]);
               }
            }
   }
}

/* build_mgh src/gh.c:1222-1365 with amr_to_mgh 1097-1165 and fill_mgh_level
 * 1171-1210, for refinement ratio 2 (no MG levels between AMR levels) */
static void build_mgh(void)
{
   plev tmp[MAXLEV];
   int in_amr[MAXLEV];
   int l, cl = MAXLEV, i, j, n, cf, num, k;
   pgrid *g, *ng;
   memset(tmp, 0, sizeof(tmp));
   memset(in_amr, 0, sizeof(in_amr));
   P.frozen = 0;
   set_tf_bits(TF_MGH_INIT);
   P.frozen = 1;
   for (l = P.n_amr; l >= P.min_level; l--) {
      cl--;
      /* replicate the AMR level (amr_to_mgh) */
      tmp[cl].dx[0] = P.amr[l].dx[0];
      tmp[cl].dx[1] = P.amr[l].dx[1];
      tmp[cl].dx[2] = P.amr[l].dx[2];
      tmp[cl].in_amrh = 1;
      in_amr[cl] = 1;
      {
         pgrid *last = 0;
         for (g = P.amr[l].grids; g; g = g->next) {
            ng = (pgrid *)calloc(1, sizeof(pgrid));
            *ng = *g;
            ng->next = 0;
            ng->coarsest = 0;
            memset(ng->own, 0, sizeof(ng->own));
            ng->own_x = 0;
            ng->gf[G_RES] = ng->gf[G_LOP] = ng->gf[G_RHS] = ng->gf[G_WRES] = 0;
            alloc_fields(ng, used_fields((1 << G_RES) | (1 << G_LOP) | (1 << G_RHS) | (1 << G_WRES)));
            if (last) last->next = ng; else tmp[cl].grids = ng;
            last = ng;
         }
      }
      if (l > P.min_level) continue;   /* rho_sp = 2: no MG levels between AMR levels */
      /* below the base: coarsen while islands allow it */
      cf = 1;
      n = -1;
      while (n) {
         double *bb, *island, *sel_island;
         cl--;
         cf *= 2;
         num = 0;
         bb = (double *)malloc(sizeof(double) * 6 * (size_t)P.sgh_num[l]);
         island = (double *)malloc(sizeof(double) * (size_t)P.sgh_num[l]);
         sel_island = (double *)malloc(sizeof(double) * (size_t)P.sgh_num[l]);
         calc_island_no(P.sgh_bbox[l], P.sgh_num[l], island, P.amr[l].dx, cf);
         for (i = 0; i < P.sgh_num[l]; i++)
            if (island[i] != 0) {
               sel_island[num] = island[i];
               for (j = 0; j < 2 * P.dim; j++) bb[2 * P.dim * num + j] = P.sgh_bbox[l][2 * i * P.dim + j];
               num++;
            }
         if (num) {
            double ldx[3];
            for (k = 0; k < 3; k++) ldx[k] = P.amr[l].dx[k] * cf;
            tmp[cl].dx[0] = ldx[0];
            tmp[cl].dx[1] = ldx[1];
            tmp[cl].dx[2] = ldx[2];
            /* fill_mgh_level + compose_cgh: each grid inserted twice in
               bbox order; the second insertion reproduces the same order */
            {
               plev first;
               memset(&first, 0, sizeof(first));
               for (i = 0; i < num; i++) {
                  double gb[6] = {0, 0, 0, 0, 0, 0};
                  for (j = 0; j < 2 * P.dim; j++) gb[j] = bb[2 * P.dim * i + j];
                  ng = new_grid(gb, ldx);
                  ng->coarsest = sel_island[i] < 0;
                  /* fill_mgh_level shape (gh.c:1198) then compose_cgh bbox */
                  insert_grid(&first, ng);
               }
               for (ng = first.grids; ng;) {
                  pgrid *nx = ng->next;
                  ng->next = 0;
                  alloc_fields(ng, used_fields((1 << NGF) - 1));
                  insert_grid(&tmp[cl], ng);
                  ng = nx;
               }
            }
            /* PAMR_inject(cl+2,1,MGH) with the frozen MGH_INIT bits */
            communicate(&tmp[cl + 1], &tmp[cl], 1, 0);
         }
         free(bb);
         free(island);
         free(sel_island);
         if (!num) {
            cl++;   /* the level was not created */
            n = 0;
         }
      }
   }
   P.n_mg = MAXLEV - cl;
   for (i = 1; i <= P.n_mg; i++) {
      P.mg[i] = tmp[cl + i - 1];
      P.mg[i].in_amrh = in_amr[cl + i - 1];
   }
   for (g = P.mg[1].grids; g; g = g->next) g->coarsest = 1;
   P.frozen = 0;
}

static void destroy_mgh(void)
{
   int l, h;
   for (l = 1; l <= P.n_mg; l++) {
      pgrid *g = P.mg[l].grids;
      while (g) {
         pgrid *n = g->next;
         for (h = 0; h < NGF; h++) if (g->own[h]) free(g->gf[h]);
         if (g->own_x) for (h = 0; h < P.dim; h++) free(g->x[h]);
         free(g);
         g = n;
      }
      P.mg[l].grids = 0;
   }
   P.n_mg = 0;
}

/* ----------------------------------------------------------- mg.c part -- */
static int grid_index(plev *lev, pgrid *g)
{
   int i = 0;
   pgrid *q;
   for (q = lev->grids; q && q != g; q = q->next) i++;
   return i;
}

static void hook_log(int kind, int L, int idx, double norm)
{
   port_result *r = P.r;
   if (!r || r->hk_n >= r->hk_cap) return;
   r->hk_kind[r->hk_n] = kind;
   r->hk_L[r->hk_n] = L;
   r->hk_idx[r->hk_n] = idx;
   r->hk_norm[r->hk_n] = norm;
   r->hk_n++;
}

static void to_ogrid(pgrid *g, oracle_grid *o)
{
   int d;
   o->dim = g->dim;
   for (d = 0; d < 3; d++) {
      o->shape[d] = g->shape[d];
      o->dx[d] = d < g->dim ? g->x[d][1] - g->x[d][0] : 1;
   }
}

/* call_rr_app amrd/util.c:73-103 with the relax (kind 0) or residual (1) hook */
static double call_rr_app(int kind, int L, int comm_only)
{
   int first = 1;
   double res = 0, lres = 0;
   pgrid *g;
   oracle_grid o;
   for (g = P.mg[L].grids; g; g = g->next) {
      if (g->comm || !comm_only) {
         double *sv[4] = {g->gf[G_SRC], g->gf[G_SRC1], g->gf[G_SRC2], g->gf[G_SRC3]};
         to_ogrid(g, &o);
         if (kind == 0)
            res = oracle_relax(P.c->pde, &o, g->gf[G_U], g->gf[G_RHS], (const double *const *)sv, g->gf[G_CMASK]);
         else
            res = oracle_residual(P.c->pde, &o, g->gf[G_RES], g->gf[G_RHS], g->gf[G_U],
                                  (const double *const *)sv, g->gf[G_CMASK]);
         hook_log(kind, L, grid_index(&P.mg[L], g), res);
         if (first) lres = res;
         lres = dmax(res, lres);
         first = 0;
      }
   }
   return lres;
}

static void call_lop(int L)   /* call_app(app_L_op) amrd/util.c:39-50 */
{
   pgrid *g;
   oracle_grid o;
   for (g = P.mg[L].grids; g; g = g->next) {
      to_ogrid(g, &o);
      double *sv[4] = {g->gf[G_SRC], g->gf[G_SRC1], g->gf[G_SRC2], g->gf[G_SRC3]};
      oracle_lop(P.c->pde, &o, g->gf[G_LOP], g->gf[G_U], (const double *const *)sv, g->gf[G_CMASK]);
      hook_log(2, L, grid_index(&P.mg[L], g), 0);
   }
}

static void clear_MG_vars(int L)   /* amrd/mg.c:242-262 */
{
   pgrid *g;
   long j;
   for (g = P.mg[L].grids; g; g = g->next)
      for (j = 0; j < gsize(g); j++) g->gf[G_RES][j] = g->gf[G_RHS][j] = g->gf[G_LOP][j] = 0;
}

static void compute_MG_rhs(int L)   /* amrd/mg.c:271-314, save_tre = 0 */
{
   pgrid *g;
   long j;
   for (g = P.mg[L].grids; g; g = g->next)
      for (j = 0; j < gsize(g); j++) {
         if (g->gf[G_CMASK][j] == CMASK_ON)
            g->gf[G_RHS][j] = -g->gf[G_RES][j] * P.c->w0_r + g->gf[G_LOP][j];
         else
            g->gf[G_RHS][j] = 0;
         g->gf[G_LOP][j] = g->gf[G_U][j];
      }
}

static void compute_cgc(int L)   /* amrd/mg.c:323-355 */
{
   pgrid *g;
   long j;
   for (g = P.mg[L - 1].grids; g; g = g->next)
      for (j = 0; j < gsize(g); j++)
         g->gf[G_RES][j] = (g->gf[G_U][j] - g->gf[G_LOP][j]) / P.c->w0_i;
   pamr_interp(L - 1);
   for (g = P.mg[L].grids; g; g = g->next)
      for (j = 0; j < gsize(g); j++) g->gf[G_U][j] += g->gf[G_RES][j];
}

static void g_dx(pgrid *g, double *dx)   /* mg_ldptr amrd/mg.c:220: x[2]-x[1] */
{
   int d;
   for (d = 0; d < 3; d++) dx[d] = d < g->dim ? g->x[d][2] - g->x[d][1] : 0;
}

/* amrd/mg.c:362-426 */
static void set_cmask_child(int L)
{
   pgrid *g, *c;
   long j;
   int is, js, ks, ie, je, ke, i, k;
   double dx[3], *mask;
   const double *bb = P.bbox;
   for (g = P.mg[L].grids; g; g = g->next) {
      mask = g->gf[G_CMASK];
      g_dx(g, dx);
      for (j = 0; j < gsize(g); j++) mask[j] = CMASK_OFF;
      if (L + 1 > P.n_mg) continue;
      for (c = P.mg[L + 1].grids; c; c = c->next) {
         const double *cb = c->bbox;
         int jj;
         js = je = ks = ke = 0;
         is = (int)dmax((cb[0] - g->bbox[0]) / dx[0] + 0.5, 0);
         ie = (int)dmin((cb[1] - g->bbox[0]) / dx[0] + 0.5, g->shape[0] - 1);
         if (is > 0 || (g->bbox[0] - bb[0]) > dx[0] / 2) is++;
         if (ie < (g->shape[0] - 1) || (bb[1] - g->bbox[1]) > dx[0] / 2) ie--;
         if (g->dim > 1) {
            js = (int)dmax((cb[2] - g->bbox[2]) / dx[1] + 0.5, 0);
            je = (int)dmin((cb[3] - g->bbox[2]) / dx[1] + 0.5, g->shape[1] - 1);
            if (js > 0 || (g->bbox[2] - bb[2]) > dx[1] / 2) js++;
            if (je < (g->shape[1] - 1) || (bb[3] - g->bbox[3]) > dx[1] / 2) je--;
            if (g->dim > 2) {
               ks = (int)dmax((cb[4] - g->bbox[4]) / dx[2] + 0.5, 0);
               ke = (int)dmin((cb[5] - g->bbox[4]) / dx[2] + 0.5, g->shape[2] - 1);
               if (ks > 0 || (g->bbox[4] - bb[4]) > dx[2] / 2) ks++;
               if (ke < (g->shape[2] - 1) || (bb[5] - g->bbox[5]) > dx[2] / 2) ke--;
            }
         }
         if (is >= 0 && js >= 0 && ks >= 0 && is <= ie && js <= je && ks <= ke &&
             ie < g->shape[0] && je < g->shape[1] && ke < g->shape[2])
            for (i = is; i <= ie; i++)
               for (jj = js; jj <= je; jj++)
                  for (k = ks; k <= ke; k++)
                     mask[i + jj * (long)g->shape[0] + k * (long)g->shape[0] * g->shape[1]] = CMASK_ON;
      }
   }
}

/* amrd/mg.c:432-488 */
static void set_cmask_bdy(int L)
{
   pgrid *g;
   long j;
   int is, js, ks, ie, je, ke, i, k;
   double dx[3], *mask;
   const double *bb = P.bbox;
   for (g = P.mg[L].grids; g; g = g->next) {
      int jj;
      mask = g->gf[G_CMASK];
      g_dx(g, dx);
      for (j = 0; j < gsize(g); j++) mask[j] = CMASK_OFF;
      is = js = ks = je = ke = 0;
      ie = g->shape[0] - 1;
      if ((g->bbox[0] - bb[0]) > dx[0] / 2) is++;
      if ((bb[1] - g->bbox[1]) > dx[0] / 2) ie--;
      if (g->dim > 1) {
         je = g->shape[1] - 1;
         if ((g->bbox[2] - bb[2]) > dx[1] / 2) js++;
         if ((bb[3] - g->bbox[3]) > dx[1] / 2) je--;
         if (g->dim > 2) {
            ke = g->shape[2] - 1;
            if ((g->bbox[4] - bb[4]) > dx[2] / 2) ks++;
            if ((bb[5] - g->bbox[5]) > dx[2] / 2) ke--;
         }
      }
      if (is >= 0 && js >= 0 && ks >= 0 && is <= ie && js <= je && ks <= ke &&
          ie < g->shape[0] && je < g->shape[1] && ke < g->shape[2])
         for (i = is; i <= ie; i++)
            for (jj = js; jj <= je; jj++)
               for (k = ks; k <= ke; k++)
                  mask[i + jj * (long)g->shape[0] + k * (long)g->shape[0] * g->shape[1]] = CMASK_ON;
   }
}

static int is_coarsest(int L)   /* amrd/mg.c:553-567 */
{
   pgrid *g;
   for (g = P.mg[L].grids; g; g = g->next) if (g->coarsest) return 1;
   return 0;
}

/* vcycle amrd/mg.c:84-201 */
static double vcycle(void)
{
   int L, Lf = P.n_mg, iter, bw;
   double res[MAXLEV + 1], ctol;
   const port_case *c = P.c;
   clear_MG_vars(Lf);
   for (L = Lf; L > 0; L--) {
      if (L < Lf) {
         res[L + 1] = call_rr_app(1, L + 1, 0);
         /* set_res_sync: freeze, clear, sync u_res only (amrd/mg.c:606-616) */
         P.frozen = 1;
         memset(P.tf, 0, sizeof(P.tf));
         P.tf[G_RES] = 1;
         pamr_sync(L + 1, 0);
         P.frozen = 0;
         clear_MG_vars(L);
         pamr_inject(L + 1);
         pamr_sync(L, 0);
         set_cmask_child(L);
         call_lop(L);
         compute_MG_rhs(L);
      }
      set_cmask_bdy(L);
      for (iter = 0; iter < c->pre_swp; iter++) {
         res[L] = call_rr_app(0, L, 0);
         bw = iter == 0 ? 0 : 1;
         pamr_sync(L, bw);
      }
   }
   for (L = 1; L <= Lf; L++) {
      ctol = res[L] * c->crtol;
      if (L > 1) compute_cgc(L);
      for (iter = 0; iter < c->pst_swp; iter++) {
         res[L] = call_rr_app(0, L, 0);
         bw = iter == 0 ? 0 : 1;
         pamr_sync(L, bw);
      }
      if (is_coarsest(L)) {
         pgrid *g;
         res[L] = ctol + 1;
         for (g = P.mg[L].grids; g; g = g->next) g->comm = g->coarsest;   /* set_comm_coarsest */
         while (iter < c->max_citer && res[L] > ctol) {
            res[L] = call_rr_app(0, L, 1);
            pamr_sync(L, 1);
            iter++;
         }
         for (g = P.mg[L].grids; g; g = g->next) g->comm = 1;              /* reset_comm */
      }
      if (L == Lf) res[Lf] = call_rr_app(1, L, 0);
   }
   return res[Lf];
}

/* --------------------------------------------------------------- entry -- */
static int same_bbox(const double *a, const double *b, int dim)
{
   int i;
   for (i = 0; i < 2 * dim; i++)
      if (fabs(a[i] - b[i]) > 1e-9 * (1 + fabs(a[i]))) return 0;
   return 1;
}

/* the AMR hierarchy of c with u and the sources filled in (PAMR_compose_hierarchy
 * plus the application's data); 0 on success */
static int port_compose(const port_case *c, port_result *r)
{
   int i, l, d;
   pgrid *g;
   if (c->dim < 2 || c->dim > 3 || c->ngrids < 1) return 1;
   memset(&P, 0, sizeof(P));
   P.c = c;
   P.r = r;
   P.dim = c->dim;
   memcpy(P.bbox, c->base_bbox, sizeof(P.bbox));
   for (i = 0; i < c->ngrids; i++) P.n_amr = imax(P.n_amr, c->lev[i]);
   if (P.n_amr >= MAXLEV - 12) return 1;
   P.min_level = c->min_level > 0 ? c->min_level : 1;
   if (P.min_level > P.n_amr) return 1;
   /* level spacing: recalc_lev_info src/gh.c:54-81, ratio 2 */
   for (d = 0; d < 3; d++) {
      P.amr_dx[1][d] = d < P.dim ? (c->base_bbox[2 * d + 1] - c->base_bbox[2 * d]) / (c->base_shape[d] - 1) : 0;
      for (l = 2; l <= P.n_amr; l++) P.amr_dx[l][d] = P.amr_dx[l - 1][d] / 2;
   }
   P.sgh_bbox = (double **)calloc((size_t)P.n_amr + 1, sizeof(double *));
   P.sgh_num = (int *)calloc((size_t)P.n_amr + 1, sizeof(int));
   for (l = 1; l <= P.n_amr; l++) {
      for (d = 0; d < 3; d++) P.amr[l].dx[d] = P.amr_dx[l][d];
      P.amr[l].in_amrh = 1;
      P.sgh_bbox[l] = (double *)malloc(sizeof(double) * 6 * (size_t)c->ngrids);
      /* save_sgh_bboxes src/gh.c:273-301; build_sgh + compose_cgh insertion */
      {
         plev first;
         memset(&first, 0, sizeof(first));
         for (i = 0; i < c->ngrids; i++)
            if (c->lev[i] == l) {
               for (d = 0; d < 2 * P.dim; d++)
                  P.sgh_bbox[l][2 * P.dim * P.sgh_num[l] + d] = c->bbox[6 * i + d];
               P.sgh_num[l]++;
               g = new_grid(&c->bbox[6 * i], P.amr[l].dx);
               insert_grid(&first, g);
            }
         for (g = first.grids; g;) {
            pgrid *nx = g->next;
            g->next = 0;
            alloc_fields(g, used_fields((1 << G_SRC) | (1 << G_U) | (1 << G_CMASK) | (1 << G_SRC1) |
                                        (1 << G_SRC2) | (1 << G_SRC3) | (1 << G_W)));
            insert_grid(&P.amr[l], g);
            g = nx;
         }
      }
   }
   /* fill u and the source from the input grids */
   for (i = 0; i < c->ngrids; i++) {
      pgrid *m = 0;
      for (g = P.amr[c->lev[i]].grids; g; g = g->next)
         if (same_bbox(g->bbox, &c->bbox[6 * i], P.dim)) m = g;
      if (!m) return 2;
      memcpy(m->gf[G_U], c->u[i], sizeof(double) * (size_t)gsize(m));
      memcpy(m->gf[G_SRC], c->src[i], sizeof(double) * (size_t)gsize(m));
      for (d = 1; d < oracle_nsrc(c->pde); d++)
         memcpy(m->gf[G_SRCK(d)], c->srcx[d - 1][i], sizeof(double) * (size_t)gsize(m));
   }
   return 0;
}

/* frees the AMR hierarchy */
static void port_free(void)
{
   int l;
   pgrid *g;
   for (l = 1; l <= P.n_amr; l++) {
      g = P.amr[l].grids;
      while (g) {
         pgrid *n = g->next;
         int h;
         for (h = 0; h < NGF; h++) if (g->own[h]) free(g->gf[h]);
         for (h = 0; h < P.dim; h++) free(g->x[h]);
         free(g);
         g = n;
      }
      free(P.sgh_bbox[l]);
   }
   free(P.sgh_bbox);
   free(P.sgh_num);
}

int port_solve(const port_case *c, port_result *r)
{
   int i, it, rc;
   double res;
   pgrid *g;
   if ((rc = port_compose(c, r))) return rc;
   /* solve_elliptics amrd/mg.c:20-79 */
   build_mgh();
   if (r) r->n_levels = P.n_mg;
   res = c->tol + 1;
   it = 0;
   while ((it < c->min_iter || res > c->tol) && it < c->max_iter) {
      res = vcycle();
      if (r && r->res) r->res[it] = res;
      it++;
   }
   if (r) r->iters = it;
   destroy_mgh();

   for (i = 0; i < c->ngrids; i++) {
      for (g = P.amr[c->lev[i]].grids; g; g = g->next)
         if (same_bbox(g->bbox, &c->bbox[6 * i], P.dim))
            memcpy(c->u[i], g->gf[G_U], sizeof(double) * (size_t)gsize(g));
   }
   port_free();
   return 0;
}
