/*
 * Hierarchy and transfer-plan builder (see pgb_plan.h).
 *
 * The geometry is reproduced bit for bit: grid ordering (insert_grid,
 * src/gh.c:235-257), shapes and bounding boxes (build_sgh src/gh.c:308-390,
 * compose_cgh src/gh.c:602-933 at one rank), MG coarsening (build_mgh
 * src/gh.c:1222-1365 with calc_island_no 1427-1467), ownership and segment
 * algebra (src/transfer.c:132-540) and the index arithmetic of
 * local_transfer (src/transfer.c:946-1163). Segments are kept in arrays in
 * the order the reference's linked lists would hold them, because that order
 * decides which of two overlapping transfers lands last.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "pgb_plan.h"

#define SMALL_DX 1e-20
#define MAXTMP 128
#define dmax(a, b) (((a) > (b)) ? (a) : (b))
#define dmin(a, b) (((a) < (b)) ? (a) : (b))
#define imax(a, b) ((a) > (b) ? (a) : (b))
#define imin(a, b) ((a) < (b) ? (a) : (b))

static int fuzz_eq(double a, double b, double f) { return fabs(b - a) < f; }
static int fuzz_lt(double a, double b, double f) { return a < -f + b; }
static int fuzz_gt(double a, double b, double f) { return a > f + b; }

/* ------------------------------------------------------------ segments -- */
typedef struct { double bb[6]; int box; } seg;
typedef struct { seg *v; int n, cap; } segv;

static void sv_push(segv *s, const seg *x)
{
   if (s->n == s->cap) {
      s->cap = s->cap ? 2 * s->cap : 16;
      s->v = (seg *)realloc(s->v, sizeof(seg) * (size_t)s->cap);
   }
   s->v[s->n++] = *x;
}
static void sv_free(segv *s) { free(s->v); s->v = 0; s->n = s->cap = 0; }

typedef struct {
   pgb_hier *h;
   int dim;
} ctx;

static double box_dx(const pgb_hbox *b, int d)
{
   return b->shape[d] > 1 ? (b->bbox[2 * d + 1] - b->bbox[2 * d]) / (b->shape[d] - 1) : SMALL_DX;
}

/* calc_gs_ibbox src/transfer.c:73-95 */
static void ibbox_of(const pgb_hier *h, const seg *s, int *ib, double *dx)
{
   const pgb_hbox *g = &h->boxes[s->box];
   int i;
   for (i = 0; i < h->dim; i++) {
      if (g->shape[i] > 1) {
         dx[i] = (g->bbox[2 * i + 1] - g->bbox[2 * i]) / (g->shape[i] - 1);
         ib[2 * i] = (int)((s->bb[2 * i] - g->bbox[2 * i]) / dx[i] + 1.01);
         ib[2 * i + 1] = (int)((s->bb[2 * i + 1] - g->bbox[2 * i]) / dx[i] + 1.99);
      } else {
         ib[2 * i] = ib[2 * i + 1] = 1;
         dx[i] = SMALL_DX;
      }
   }
}

/* alloc_gsl src/transfer.c:132-188 (no ghost zones at one rank, not periodic);
 * returns 0 when the segment is empty */
static int seg_of_box(const pgb_hier *h, int box, int interior, int reduce, seg *out)
{
   const pgb_hbox *g = &h->boxes[box];
   int i, ib[6];
   double dx, dxt[3];
   memset(out, 0, sizeof(*out));
   out->box = box;
   for (i = 0; i < h->dim; i++) {
      dx = box_dx(g, i);
      out->bb[2 * i] = g->bbox[2 * i];
      out->bb[2 * i + 1] = g->bbox[2 * i + 1];
      if (reduce > 0) {
         if (fuzz_gt(out->bb[2 * i], h->base_bbox[2 * i], dx / 2)) out->bb[2 * i] += reduce * dx;
         if (fuzz_lt(out->bb[2 * i + 1], h->base_bbox[2 * i + 1], dx / 2))
            out->bb[2 * i + 1] += -reduce * dx;
      }
      if (interior || reduce) {
         ibbox_of(h, out, ib, dxt);
         if ((ib[2 * i + 1] - ib[2 * i] + 1) < 1) return 0;
      }
   }
   return 1;
}

/* gs_subtract src/transfer.c:218-285: pieces of A outside B, appended to out
 * in the order the reference's prepending list ends up in */
static void gs_subtract(const pgb_hier *h, const seg *A, const seg *B, segv *out)
{
   double cut[6], dx[3];
   seg pieces[6];
   int np = 0, d = h->dim, i, j;
   const pgb_hbox *g = &h->boxes[A->box];
   for (i = 0; i < d; i++) {
      cut[2 * i] = A->bb[2 * i];
      cut[2 * i + 1] = A->bb[2 * i + 1];
      dx[i] = box_dx(g, i);
      if (fuzz_gt(B->bb[2 * i], A->bb[2 * i + 1], dx[i] / 2) ||
          fuzz_gt(A->bb[2 * i], B->bb[2 * i + 1], dx[i] / 2)) {
         sv_push(out, A);
         return;
      }
   }
   for (i = 0; i < d; i++) {
      cut[2 * i] = dmax(A->bb[2 * i], B->bb[2 * i]);
      if (fuzz_gt(cut[2 * i], A->bb[2 * i], dx[i] / 2)) {
         seg *c = &pieces[np++];
         *c = *A;
         for (j = 0; j < d; j++) {
            if (i == j) {
               c->bb[2 * i] = A->bb[2 * i];
               c->bb[2 * i + 1] = dmax(c->bb[2 * i], cut[2 * i] - dx[i]);
            } else {
               c->bb[2 * j] = cut[2 * j];
               c->bb[2 * j + 1] = cut[2 * j + 1];
            }
         }
      }
      cut[2 * i + 1] = dmin(A->bb[2 * i + 1], B->bb[2 * i + 1]);
      if (fuzz_lt(cut[2 * i + 1], A->bb[2 * i + 1], dx[i] / 2)) {
         seg *c = &pieces[np++];
         *c = *A;
         for (j = 0; j < d; j++) {
            if (i == j) {
               c->bb[2 * i + 1] = A->bb[2 * i + 1];
               c->bb[2 * i] = dmin(c->bb[2 * i + 1], cut[2 * i + 1] + dx[i]);
            } else {
               c->bb[2 * j] = cut[2 * j];
               c->bb[2 * j + 1] = cut[2 * j + 1];
            }
         }
      }
   }
   for (i = np - 1; i >= 0; i--) sv_push(out, &pieces[i]);
}

/* gsl_subtract src/transfer.c:287-314 (A is one segment) */
static void gsl_subtract(const pgb_hier *h, const seg *A, const segv *B, segv *out)
{
   segv C = {0, 0, 0}, C0;
   int b, c;
   sv_push(&C, A);
   for (b = 0; b < B->n; b++) {
      memset(&C0, 0, sizeof(C0));
      for (c = 0; c < C.n; c++) gs_subtract(h, &C.v[c], &B->v[b], &C0);
      sv_free(&C);
      C = C0;
   }
   for (c = 0; c < C.n; c++) sv_push(out, &C.v[c]);
   sv_free(&C);
}

static int box_in_comm(const pgb_hier *h, int box, int comm_mode)
{
   return comm_mode == 0 || h->boxes[box].coarsest;
}

/* build_owned_gsl src/transfer.c:415-458 */
static void build_owned(const pgb_hier *h, const pgb_hlevel *lev, int interior, int extend,
                        int comm_mode, segv *owned)
{
   segv ints = {0, 0, 0};
   int cint = interior ? 1 : 0, cred = interior > 1 ? interior - 1 : 0, b, i;
   seg s;
   for (b = 0; b < lev->nbox; b++) {
      if (!box_in_comm(h, lev->box[b], comm_mode)) continue;
      if (!seg_of_box(h, lev->box[b], cint, cred, &s)) continue;
      gsl_subtract(h, &s, &ints, owned);
      sv_push(&ints, &s);
   }
   sv_free(&ints);
   if (extend)   /* extend_gsl src/transfer.c:364-386 */
      for (b = 0; b < owned->n; b++) {
         const pgb_hbox *g = &h->boxes[owned->v[b].box];
         for (i = 0; i < h->dim; i++)
            if (g->shape[i] > 1) {
               double dx = (g->bbox[2 * i + 1] - g->bbox[2 * i]) / (g->shape[i] - 1);
               owned->v[b].bb[2 * i] = dmax(owned->v[b].bb[2 * i] - dx, g->bbox[2 * i]);
               owned->v[b].bb[2 * i + 1] = dmin(owned->v[b].bb[2 * i + 1] + dx, g->bbox[2 * i + 1]);
            }
      }
}

/* build_complete_gsl src/transfer.c:465-504: every grid of the level, or
 * with AMR_bdy_only > 0 the band of that width along the grids' AMR
 * boundaries: the union minus each grid shrunk by the width away from the
 * physical boundary, subtracted grid by grid as gsl_subtract
 * (src/transfer.c:287-314) orders the pieces */
static void build_complete(const pgb_hier *h, const pgb_hlevel *lev, int comm_mode, int amr_bdy_only, segv *out)
{
   int b, c;
   seg s;
   segv all = {0, 0, 0}, inner = {0, 0, 0};
   for (b = 0; b < lev->nbox; b++)
      if (box_in_comm(h, lev->box[b], comm_mode) && seg_of_box(h, lev->box[b], 0, 0, &s)) {
         sv_push(&all, &s);
         if (amr_bdy_only > 0 && seg_of_box(h, lev->box[b], 0, amr_bdy_only, &s)) sv_push(&inner, &s);
      }
   if (amr_bdy_only <= 0) {
      for (c = 0; c < all.n; c++) sv_push(out, &all.v[c]);
   } else {
      segv cur = all;
      all.v = 0;
      all.n = all.cap = 0;
      for (b = 0; b < inner.n; b++) {
         segv next = {0, 0, 0};
         for (c = 0; c < cur.n; c++) gs_subtract(h, &cur.v[c], &inner.v[b], &next);
         sv_free(&cur);
         cur = next;
      }
      for (c = 0; c < cur.n; c++) sv_push(out, &cur.v[c]);
      sv_free(&cur);
   }
   sv_free(&all);
   sv_free(&inner);
}

/* gs_and src/transfer.c:325-356 */
static int gs_and(const pgb_hier *h, const seg *A, const seg *B, seg *A0, seg *B0)
{
   double nb[6] = {0, 0, 0, 0, 0, 0};
   int i;
   for (i = 0; i < h->dim; i++) {
      double dxm = dmax(box_dx(&h->boxes[A->box], i), box_dx(&h->boxes[B->box], i));
      nb[2 * i] = dmax(A->bb[2 * i], B->bb[2 * i]);
      nb[2 * i + 1] = dmin(A->bb[2 * i + 1], B->bb[2 * i + 1]);
      if (fuzz_lt(nb[2 * i + 1], nb[2 * i], dxm / 2)) return 0;
   }
   *A0 = *A;
   *B0 = *B;
   for (i = 0; i < h->dim; i++) {
      A0->bb[2 * i] = B0->bb[2 * i] = nb[2 * i];
      A0->bb[2 * i + 1] = B0->bb[2 * i + 1] = nb[2 * i + 1];
   }
   return 1;
}

/* build_gstl src/transfer.c:514-540 */
static void build_pairs(const pgb_hier *h, const segv *src, const segv *dst, segv *ps, segv *pd)
{
   int a, b;
   seg s, d;
   for (a = 0; a < src->n; a++)
      for (b = 0; b < dst->n; b++) {
         if (src->v[a].box == dst->v[b].box) continue;
         if (gs_and(h, &src->v[a], &dst->v[b], &s, &d)) {
            sv_push(ps, &s);
            sv_push(pd, &d);
         }
      }
}

/* calc_delta src/transfer.c:545-575 */
static int calc_delta(const pgb_hier *h, const seg *src, const seg *dst, int *irho)
{
   double dxsm = 0, dxdm = 0;
   int i;
   const pgb_hbox *gs = &h->boxes[src->box], *gd = &h->boxes[dst->box];
   *irho = 0;
   for (i = 0; i < h->dim; i++)
      if (gs->shape[i] > 1 && gd->shape[i] > 1) {
         dxsm = dmax(dxsm, (gs->bbox[2 * i + 1] - gs->bbox[2 * i]) / (gs->shape[i] - 1));
         dxdm = dmax(dxdm, (gd->bbox[2 * i + 1] - gd->bbox[2 * i]) / (gd->shape[i] - 1));
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

/* align_src_bbox src/transfer.c:101-121 */
static void align_src(const pgb_hier *h, seg *src, seg *dst)
{
   int i;
   const pgb_hbox *gs = &h->boxes[src->box], *gd = &h->boxes[dst->box];
   for (i = 0; i < h->dim; i++)
      if (gs->shape[i] > 1 && gd->shape[i] > 1) {
         double dxs = (gs->bbox[2 * i + 1] - gs->bbox[2 * i]) / (gs->shape[i] - 1);
         double dxd = (gd->bbox[2 * i + 1] - gd->bbox[2 * i]) / (gd->shape[i] - 1);
         src->bb[2 * i] = ((int)((src->bb[2 * i] - gd->bbox[2 * i] + dxs / 2) / dxd)) * dxd + gd->bbox[2 * i];
         if (fuzz_lt(src->bb[2 * i], gs->bbox[2 * i], dxs / 2)) src->bb[2 * i] += dxd;
         dst->bb[2 * i] = src->bb[2 * i];
         src->bb[2 * i + 1] =
            ((int)((src->bb[2 * i + 1] - gd->bbox[2 * i] + dxd - dxs / 2) / dxd)) * dxd + gd->bbox[2 * i];
         if (fuzz_gt(src->bb[2 * i + 1], gs->bbox[2 * i + 1], dxs / 2)) src->bb[2 * i + 1] -= dxd;
         dst->bb[2 * i + 1] = src->bb[2 * i + 1];
      }
}

/* ------------------------------------------------------------- op lists -- */
typedef struct { void *v; int n, cap; size_t sz; } opv;
static void ov_push(opv *o, const void *x)
{
   if (o->n == o->cap) {
      o->cap = o->cap ? 2 * o->cap : 16;
      o->v = realloc(o->v, o->sz * (size_t)o->cap);
   }
   memcpy((char *)o->v + o->sz * (size_t)o->n, x, o->sz);
   o->n++;
}

/* the Fortran kernels return silently when a segment leaves the array
 * (src/m_util_r8.f:31-38); such ops are dropped here */
static int in_range(int s, int n, int stride, int N) { return !(s < 1 || s + (n - 1) * stride > N); }

/* dst rectangle of an op, for batching */
typedef struct { int box, lo[3], hi[3]; } rect;

static int rect_overlap(const rect *a, const rect *b)
{
   int d;
   if (a->box != b->box) return 0;
   for (d = 0; d < 3; d++)
      if (a->hi[d] < b->lo[d] || b->hi[d] < a->lo[d]) return 0;
   return 1;
}

/* splits ops into ordered batches of pairwise disjoint destinations */
static void make_batches(pgb_plan *p, const rect *r, const long *pts)
{
   int i, j, start = 0;
   p->batch_start = (int *)malloc(sizeof(int) * (size_t)(p->nops + 1));
   p->batch_maxpts = (int *)malloc(sizeof(int) * (size_t)(p->nops + 1));
   p->nbatch = 0;
   if (p->nops == 0) {
      p->batch_start[0] = 0;
      return;
   }
   p->batch_start[0] = 0;
   p->batch_maxpts[0] = 0;
   for (i = 0; i < p->nops; i++) {
      int clash = 0;
      for (j = start; j < i && !clash; j++) clash = rect_overlap(&r[i], &r[j]);
      if (clash) {
         p->nbatch++;
         p->batch_start[p->nbatch] = i;
         p->batch_maxpts[p->nbatch] = 0;
         start = i;
      }
      if (pts[i] > p->batch_maxpts[p->nbatch]) p->batch_maxpts[p->nbatch] = (int)pts[i];
   }
   p->nbatch++;
   p->batch_start[p->nbatch] = p->nops;
}

enum { COMM_SYNC, COMM_INJECT, COMM_INTERP };

/* communicate() src/pamr.c:533-593 + local_transfer, as an op plan */
static void plan_comm_bdy(pgb_hier *h, int kind, int l1, int l2, int interior, int extend, int comm_mode,
                          int amr_bdy_only, const int *field_ops, pgb_plan *out);

static void plan_comm(pgb_hier *h, int kind, int l1, int l2, int interior, int extend,
                      int comm_mode, const int *field_ops, pgb_plan *out)
{
   plan_comm_bdy(h, kind, l1, l2, interior, extend, comm_mode, 0, field_ops, out);
}

/* communicate (src/pamr.c:533-593) as a flat op list, for one transfer kind */
static void plan_comm_bdy(pgb_hier *h, int kind, int l1, int l2, int interior, int extend, int comm_mode,
                          int amr_bdy_only, const int *field_ops, pgb_plan *out)
{
   segv src = {0, 0, 0}, dst = {0, 0, 0}, ps = {0, 0, 0}, pd = {0, 0, 0};
   opv ops = {0, 0, 0, 0};
   rect *rects;
   long *pts;
   int p, f, any = 0;
   memset(out, 0, sizeof(*out));
   if (field_ops)
      for (f = 0; f < PGB_NF; f++) any |= field_ops[f];
   if (kind == COMM_SYNC) ops.sz = sizeof(pgb_copy_op);
   else if (kind == COMM_INJECT) ops.sz = sizeof(pgb_restrict_op);
   else ops.sz = sizeof(pgb_interp_op);
   build_owned(h, &h->lev[l1], interior, extend, comm_mode, &src);
   build_complete(h, &h->lev[l2], comm_mode, amr_bdy_only, &dst);
   build_pairs(h, &src, &dst, &ps, &pd);
   rects = (rect *)malloc(sizeof(rect) * (size_t)(ps.n + 1));
   pts = (long *)malloc(sizeof(long) * (size_t)(ps.n + 1));
   for (p = 0; p < ps.n; p++) {
      seg *s = &ps.v[p], *d = &pd.v[p];
      const pgb_hbox *g1 = &h->boxes[s->box], *g2 = &h->boxes[d->box];
      int irho, delta = calc_delta(h, s, d, &irho), ib[6] = {1, 1, 1, 1, 1, 1}, ibd[6] = {1, 1, 1, 1, 1, 1};
      double dx[3], dxd[3];
      int n1[3] = {1, 1, 1}, n2[3] = {1, 1, 1}, a1[3] = {1, 1, 1}, a2[3] = {1, 1, 1};
      int ns[3] = {1, 1, 1}, nd[3] = {1, 1, 1}, d_;
      rect r;
      if (delta == 1) align_src(h, s, d);
      ibbox_of(h, s, ib, dx);
      ibbox_of(h, d, ibd, dxd);
      for (d_ = 0; d_ < h->dim; d_++) {
         a1[d_] = ib[2 * d_];
         a2[d_] = ibd[2 * d_];
         ns[d_] = ib[2 * d_ + 1] - ib[2 * d_] + 1;
         nd[d_] = ibd[2 * d_ + 1] - ibd[2 * d_] + 1;
         n1[d_] = g1->shape[d_];
         n2[d_] = g2->shape[d_];
      }
      r.box = d->box;
      if (kind == COMM_SYNC) {
         pgb_copy_op o;
         if (delta != 0) continue;
         for (d_ = 0; d_ < 3; d_++)
            if (!in_range(a1[d_], ns[d_], 1, n1[d_]) || !in_range(a2[d_], ns[d_], 1, n2[d_])) break;
         if (d_ < 3) continue;
         o.src_box = s->box; o.dst_box = d->box;
         o.i1 = a1[0]; o.j1 = a1[1]; o.k1 = a1[2];
         o.i2 = a2[0]; o.j2 = a2[1]; o.k2 = a2[2];
         o.ni = ns[0]; o.nj = ns[1]; o.nk = ns[2];
         for (d_ = 0; d_ < 3; d_++) { r.lo[d_] = a2[d_]; r.hi[d_] = a2[d_] + ns[d_] - 1; }
         pts[ops.n] = (long)ns[0] * ns[1] * ns[2];
         rects[ops.n] = r;
         ov_push(&ops, &o);
      } else if (kind == COMM_INJECT) {
         pgb_restrict_op o;
         if (delta != 1 || !any) continue;
         for (d_ = 0; d_ < 3; d_++)
            if (!in_range(a1[d_], nd[d_], irho, n1[d_]) || !in_range(a2[d_], nd[d_], 1, n2[d_])) break;
         if (d_ < 3) continue;
         memset(&o, 0, sizeof(o));
         o.src_box = s->box; o.dst_box = d->box;
         o.i1 = a1[0]; o.j1 = a1[1]; o.k1 = a1[2];
         o.i2 = a2[0]; o.j2 = a2[1]; o.k2 = a2[2];
         o.ni = nd[0]; o.nj = nd[1]; o.nk = nd[2];
         o.irho = irho;
         for (f = 0; f < PGB_NF; f++) o.op[f] = field_ops[f];
         for (d_ = 0; d_ < 3; d_++) { r.lo[d_] = a2[d_]; r.hi[d_] = a2[d_] + nd[d_] - 1; }
         pts[ops.n] = (long)nd[0] * nd[1] * nd[2];
         rects[ops.n] = r;
         ov_push(&ops, &o);
      } else {
         pgb_interp_op o;
         int bl = h->prm.interp_buffer, w1[3] = {1, 1, 1}, wn[3] = {1, 1, 1}, wb[3] = {1, 1, 1};
         int wlen[3] = {1, 1, 1};
         if (delta != -1 || !any) continue;
         for (d_ = 0; d_ < h->dim; d_++) {
            int b2 = (int)((s->bb[2 * d_] - g1->bbox[2 * d_]) / dxd[d_] + 1.5);
            int i2i = imax(1, (((b2 - 1) / irho) - bl) * irho + 1);
            int i1i = (i2i - 1) / irho + 1;
            int nii = imin(n1[d_], (b2 + nd[d_] - 1) / irho + 1 + bl + 1) - i1i + 1;
            w1[d_] = i1i;
            wn[d_] = nii;
            wlen[d_] = (nii - 1) * irho + 1;
            wb[d_] = b2 - i2i + 1;
         }
         /* dminterp3d's own range check (m_util_r8.f:488-495), then the
            window -> grid copy's (m_util_r8.f:31-38) */
         for (d_ = 0; d_ < 3; d_++)
            if (!in_range(w1[d_], wn[d_], 1, n1[d_])) break;
         if (d_ < 3) {
            snprintf(h->err, sizeof(h->err), "interpolation window outside the coarse grid");
            continue;
         }
         for (d_ = 0; d_ < 3; d_++)
            if (!in_range(wb[d_], nd[d_], 1, wlen[d_]) || !in_range(a2[d_], nd[d_], 1, n2[d_])) break;
         if (d_ < 3) continue;
         o.src_box = s->box; o.dst_box = d->box;
         o.i1i = w1[0]; o.j1i = w1[1]; o.k1i = w1[2];
         o.nii = wn[0]; o.nji = wn[1]; o.nki = wn[2];
         o.i2b = wb[0]; o.j2b = wb[1]; o.k2b = wb[2];
         o.i2 = a2[0]; o.j2 = a2[1]; o.k2 = a2[2];
         o.nib = nd[0]; o.njb = nd[1]; o.nkb = nd[2];
         o.irho = irho;
         o.ord = field_ops[PGB_F_RES];
         for (d_ = 0; d_ < 3; d_++) { r.lo[d_] = a2[d_]; r.hi[d_] = a2[d_] + nd[d_] - 1; }
         pts[ops.n] = (long)nd[0] * nd[1] * nd[2];
         rects[ops.n] = r;
         ov_push(&ops, &o);
      }
   }
   out->nops = ops.n;
   out->h_ops = ops.v;
   make_batches(out, rects, pts);
   free(rects);
   free(pts);
   sv_free(&src);
   sv_free(&dst);
   sv_free(&ps);
   sv_free(&pd);
}

/* ----------------------------------------------------------- hierarchy -- */
/* insert_grid src/gh.c:235-257 on an index list */
static void insert_sorted(const pgb_hier *h, int *list, int *n, int box)
{
   const double *g = h->boxes[box].bbox;
   int dim = h->dim, pos = 0, i;
   while (pos < *n) {
      const double *c = h->boxes[list[pos]].bbox;
      if ((c[0] < g[0]) && ((dim < 2) || c[2] < g[2]) && ((dim < 3) || c[4] < g[4]) &&
          (c[1] < g[1]) && ((dim < 2) || c[3] < g[3]) && ((dim < 3) || c[5] < g[5]))
         pos++;
      else
         break;
   }
   for (i = *n; i > pos; i--) list[i] = list[i - 1];
   list[pos] = box;
   (*n)++;
}

static int new_box(pgb_hier *h, const double *bbox, const double *lev_dx, int *cap)
{
   pgb_hbox *b;
   int d, m;
   if (h->nbox == *cap) {
      *cap = *cap ? 2 * *cap : 64;
      h->boxes = (pgb_hbox *)realloc(h->boxes, sizeof(pgb_hbox) * (size_t)*cap);
   }
   b = &h->boxes[h->nbox];
   memset(b, 0, sizeof(*b));
   b->amr_grid = -1;
   b->shape[0] = b->shape[1] = b->shape[2] = 1;
   for (d = 0; d < h->dim; d++) {
      int n = (int)((bbox[2 * d + 1] - bbox[2 * d]) / lev_dx[d] + 1.5);  /* gh.c:352, 1198 */
      b->shape[d] = n;
      b->bbox[2 * d] = bbox[2 * d] + lev_dx[d] * 0;                     /* gh.c:774-775 */
      b->bbox[2 * d + 1] = bbox[2 * d] + lev_dx[d] * (n - 1);
   }
   for (d = 0; d < h->dim; d++) {
      double x, dx = (b->bbox[2 * d + 1] - b->bbox[2 * d]) / (b->shape[d] - 1);
      b->x[d] = (double *)malloc(sizeof(double) * (size_t)b->shape[d]);
      for (m = 0, x = b->bbox[2 * d]; m < b->shape[d]; m++, x += dx) b->x[d][m] = x;
   }
   return h->nbox++;
}

/* calc_island_no src/gh.c:1427-1467 */
static void calc_island_no(const pgb_hier *h, const double *bb, int num, double *island,
                           const double *dx, int cf)
{
   int i, j, k, delta = 1, shape, overlap, mcw = h->prm.min_cwidth, D = h->dim;
   for (i = 0; i < num; i++) {
      island[i] = i + 1;
      for (j = 0; j < D; j++) {
         shape = (int)((bb[2 * i * D + 2 * j + 1] - bb[2 * i * D + 2 * j]) / dx[j] + 1.5);
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
               for (k = 0; k < D; k++)
                  if (fuzz_gt(bb[2 * i * D + 2 * k], bb[2 * j * D + 2 * k + 1], dx[k] / 2) ||
                      fuzz_gt(bb[2 * i * D + 2 * k + 1], bb[2 * j * D + 2 * k], dx[k] / 2))
                     overlap = 0;
               if (overlap) {
                  delta++;
                  if (island[i] == 0 || island[j] == 0) island[i] = island[j] = 0;
                  else island[i] = island[j] = dmin(island[i], island[j]);
               }
            }
   }
}

static void set_level_boxes(pgb_hlevel *lv, const int *list, int n)
{
   lv->nbox = n;
   lv->box = (int *)malloc(sizeof(int) * (size_t)(n ? n : 1));
   memcpy(lv->box, list, sizeof(int) * (size_t)n);
}

/* set_cmask_child amrd/mg.c:362-426 and set_cmask_bdy amrd/mg.c:432-488 */
static void build_masks(pgb_hier *h)
{
   int L, b, c, D = h->dim;
   const double *bb = h->base_bbox;
   for (L = 1; L <= h->nlev; L++)
      for (b = 0; b < h->lev[L].nbox; b++) {
         pgb_hbox *g = &h->boxes[h->lev[L].box[b]];
         long n = (long)g->shape[0] * g->shape[1] * g->shape[2];
         double dx[3] = {0, 0, 0};
         int is, js, ks, ie, je, ke, i, j, k, d;
         for (d = 0; d < D; d++) dx[d] = g->x[d][2] - g->x[d][1];   /* mg_ldptr, amrd/mg.c:220 */
         g->child_mask = (uint8_t *)calloc((size_t)n, 1);
         g->bdy_mask = (uint8_t *)calloc((size_t)n, 1);
         if (L < h->nlev)
            for (c = 0; c < h->lev[L + 1].nbox; c++) {
               const double *cb = h->boxes[h->lev[L + 1].box[c]].bbox;
               js = je = ks = ke = 0;
               is = (int)dmax((cb[0] - g->bbox[0]) / dx[0] + 0.5, 0);
               ie = (int)dmin((cb[1] - g->bbox[0]) / dx[0] + 0.5, g->shape[0] - 1);
               if (is > 0 || (g->bbox[0] - bb[0]) > dx[0] / 2) is++;
               if (ie < (g->shape[0] - 1) || (bb[1] - g->bbox[1]) > dx[0] / 2) ie--;
               if (D > 1) {
                  js = (int)dmax((cb[2] - g->bbox[2]) / dx[1] + 0.5, 0);
                  je = (int)dmin((cb[3] - g->bbox[2]) / dx[1] + 0.5, g->shape[1] - 1);
                  if (js > 0 || (g->bbox[2] - bb[2]) > dx[1] / 2) js++;
                  if (je < (g->shape[1] - 1) || (bb[3] - g->bbox[3]) > dx[1] / 2) je--;
                  if (D > 2) {
                     ks = (int)dmax((cb[4] - g->bbox[4]) / dx[2] + 0.5, 0);
                     ke = (int)dmin((cb[5] - g->bbox[4]) / dx[2] + 0.5, g->shape[2] - 1);
                     if (ks > 0 || (g->bbox[4] - bb[4]) > dx[2] / 2) ks++;
                     if (ke < (g->shape[2] - 1) || (bb[5] - g->bbox[5]) > dx[2] / 2) ke--;
                  }
               }
               if (is >= 0 && js >= 0 && ks >= 0 && is <= ie && js <= je && ks <= ke &&
                   ie < g->shape[0] && je < g->shape[1] && ke < g->shape[2])
                  for (i = is; i <= ie; i++)
                     for (j = js; j <= je; j++)
                        for (k = ks; k <= ke; k++)
                           g->child_mask[i + j * (long)g->shape[0] + k * (long)g->shape[0] * g->shape[1]] = 1;
            }
         is = js = ks = je = ke = 0;
         ie = g->shape[0] - 1;
         if ((g->bbox[0] - bb[0]) > dx[0] / 2) is++;
         if ((bb[1] - g->bbox[1]) > dx[0] / 2) ie--;
         if (D > 1) {
            je = g->shape[1] - 1;
            if ((g->bbox[2] - bb[2]) > dx[1] / 2) js++;
            if ((bb[3] - g->bbox[3]) > dx[1] / 2) je--;
            if (D > 2) {
               ke = g->shape[2] - 1;
               if ((g->bbox[4] - bb[4]) > dx[2] / 2) ks++;
               if ((bb[5] - g->bbox[5]) > dx[2] / 2) ke--;
            }
         }
         if (is >= 0 && js >= 0 && ks >= 0 && is <= ie && js <= je && ks <= ke &&
             ie < g->shape[0] && je < g->shape[1] && ke < g->shape[2])
            for (i = is; i <= ie; i++)
               for (j = js; j <= je; j++)
                  for (k = ks; k <= ke; k++)
                     g->bdy_mask[i + j * (long)g->shape[0] + k * (long)g->shape[0] * g->shape[1]] = 1;
         /* relax/residual visit interior points only (num.f:216-219) */
         {
            int all = 1, cnt = 0, kl = D == 3 ? 1 : 0, kh = D == 3 ? g->shape[2] - 2 : 0;
            for (k = kl; k <= kh; k++)
               for (j = 1; j <= g->shape[1] - 2; j++)
                  for (i = 1; i <= g->shape[0] - 2; i++) {
                     if (g->bdy_mask[i + j * (long)g->shape[0] + k * (long)g->shape[0] * g->shape[1]]) cnt++;
                     else all = 0;
                  }
            g->count = cnt;
            if (all) g->flags |= PGB_BOX_BDY_INTERIOR;
         }
      }
}

static int is_pow2(double v)
{
   int e;
   double m = frexp(v, &e);
   return v > 0 && m == 0.5;
}

int pgb_hier_build(pgb_hier *h, int dim, int pde, const int *base_shape, const double *base_bbox,
                   int ngrids, const int *grid_level, const double *grid_bbox,
                   const pgb_hparams *prm)
{
   int cap = 0, l, i, d, cl, nl;
   double amr_dx[PGB_MAXLEV + 1][3];
   int *tmp_list[PGB_MAXLEV + 2];
   int tmp_n[PGB_MAXLEV + 2], tmp_amr[PGB_MAXLEV + 2];
   double tmp_dx[PGB_MAXLEV + 2][3];
   int *amr_list[PGB_MAXLEV + 1], amr_n[PGB_MAXLEV + 1];
   int ops_init[PGB_NF], ops_inj[PGB_NF], ops_inj_mg[PGB_NF], ops_sync[PGB_NF], ops_int[PGB_NF];
   memset(h, 0, sizeof(*h));
   if (dim < 2 || dim > 3) { snprintf(h->err, sizeof(h->err), "dim must be 2 or 3"); return 1; }
   if (ngrids < 1) { snprintf(h->err, sizeof(h->err), "no grids"); return 1; }
   if (prm->interp_order != 2 && prm->interp_order != 4) {
      snprintf(h->err, sizeof(h->err), "interp_order must be 2 or 4");
      return 1;
   }
   h->dim = dim;
   h->pde = pde;
   h->prm = *prm;
   h->ngrids = ngrids;
   for (d = 0; d < 3; d++) h->base_shape[d] = d < dim ? base_shape[d] : 1;
   for (d = 0; d < 6; d++) h->base_bbox[d] = d < 2 * dim ? base_bbox[d] : 0;
   if (prm->min_level < 1) { snprintf(h->err, sizeof(h->err), "min_level must be >= 1"); return 1; }
   for (i = 0; i < ngrids; i++) {
      if (grid_level[i] < 1 || grid_level[i] >= PGB_MAXLEV / 2) {
         snprintf(h->err, sizeof(h->err), "grid %d: level out of range", i);
         return 1;
      }
      h->n_amr = imax(h->n_amr, grid_level[i]);
   }
   if (prm->min_level > h->n_amr) {
      snprintf(h->err, sizeof(h->err), "min_level %d above the finest level %d", prm->min_level, h->n_amr);
      return 1;
   }
   /* recalc_lev_info src/gh.c:54-81, refinement ratio 2 */
   for (d = 0; d < 3; d++) {
      amr_dx[1][d] = d < dim ? (base_bbox[2 * d + 1] - base_bbox[2 * d]) / (base_shape[d] - 1) : 0;
      for (l = 2; l <= h->n_amr; l++) amr_dx[l][d] = amr_dx[l - 1][d] / 2;
   }
   /* AMR levels: build_sgh then compose_cgh, each inserting in bbox order */
   h->grid_box = (int *)malloc(sizeof(int) * (size_t)ngrids);
   for (i = 0; i < ngrids; i++) h->grid_box[i] = -1;   /* grids below min_level stay outside */
   for (l = prm->min_level; l <= h->n_amr; l++) {
      int *first = (int *)malloc(sizeof(int) * (size_t)ngrids), nf = 0;
      amr_list[l] = (int *)malloc(sizeof(int) * (size_t)ngrids);
      amr_n[l] = 0;
      for (i = 0; i < ngrids; i++)
         if (grid_level[i] == l) {
            int b = new_box(h, &grid_bbox[6 * i], amr_dx[l], &cap);
            h->boxes[b].amr_grid = i;
            h->grid_box[i] = b;
            insert_sorted(h, first, &nf, b);
         }
      for (i = 0; i < nf; i++) insert_sorted(h, amr_list[l], &amr_n[l], first[i]);
      free(first);
      if (!amr_n[l]) { snprintf(h->err, sizeof(h->err), "AMR level %d has no grids", l); return 1; }
      for (i = 0; i < amr_n[l]; i++) {
         for (d = 0; d < dim; d++)
            if (h->boxes[amr_list[l][i]].shape[d] < 3) {
               snprintf(h->err, sizeof(h->err), "grids need at least 3 points per dimension");
               return 1;
            }
      }
   }
   /* MG hierarchy: build_mgh src/gh.c:1222-1365 */
   cl = PGB_MAXLEV + 1;
   for (l = h->n_amr; l >= prm->min_level; l--) {
      const int lmin = prm->min_level;
      cl--;
      tmp_n[cl] = amr_n[l];
      tmp_list[cl] = (int *)malloc(sizeof(int) * (size_t)amr_n[l]);
      memcpy(tmp_list[cl], amr_list[l], sizeof(int) * (size_t)amr_n[l]);
      tmp_amr[cl] = 1;
      for (d = 0; d < 3; d++) tmp_dx[cl][d] = amr_dx[l][d];
      if (l > lmin) continue;
      {
         /* below the coarsest AMR level of the MG hierarchy (build_mgh's
          * min_lev, src/gh.c:1285-1340): coarsen that level's sgh boxes */
         int cf = 1, more = 1, nsgh = 0;
         double *sgh = (double *)malloc(sizeof(double) * 2 * dim * (size_t)ngrids);
         double *island = (double *)malloc(sizeof(double) * (size_t)ngrids);
         /* save_sgh_bboxes src/gh.c:273-301: input order */
         for (i = 0; i < ngrids; i++)
            if (grid_level[i] == lmin) {
               for (d = 0; d < 2 * dim; d++) sgh[2 * dim * nsgh + d] = grid_bbox[6 * i + d];
               nsgh++;
            }
         while (more) {
            int num = 0, *first, nf = 0;
            double ldx[3];
            cf *= 2;
            calc_island_no(h, sgh, nsgh, island, amr_dx[lmin], cf);
            first = (int *)malloc(sizeof(int) * (size_t)nsgh);
            for (d = 0; d < 3; d++) ldx[d] = amr_dx[lmin][d] * cf;
            for (i = 0; i < nsgh; i++)
               if (island[i] != 0) {
                  double gb[6] = {0, 0, 0, 0, 0, 0};
                  int b;
                  for (d = 0; d < 2 * dim; d++) gb[d] = sgh[2 * dim * i + d];
                  b = new_box(h, gb, ldx, &cap);
                  h->boxes[b].coarsest = island[i] < 0;
                  insert_sorted(h, first, &nf, b);
                  num++;
               }
            if (num) {
               if (cl <= 1) { snprintf(h->err, sizeof(h->err), "too many MG levels"); return 1; }
               cl--;
               tmp_list[cl] = (int *)malloc(sizeof(int) * (size_t)num);
               tmp_n[cl] = 0;
               for (i = 0; i < nf; i++) insert_sorted(h, tmp_list[cl], &tmp_n[cl], first[i]);
               tmp_amr[cl] = 0;
               for (d = 0; d < 3; d++) tmp_dx[cl][d] = ldx[d];
            } else
               more = 0;
            free(first);
         }
         free(sgh);
         free(island);
      }
   }
   nl = PGB_MAXLEV + 1 - cl;
   h->nlev = nl;
   for (i = 1; i <= nl; i++) {
      pgb_hlevel *lv = &h->lev[i];
      int b;
      set_level_boxes(lv, tmp_list[cl + i - 1], tmp_n[cl + i - 1]);
      free(tmp_list[cl + i - 1]);
      lv->in_amrh = tmp_amr[cl + i - 1];
      for (d = 0; d < 3; d++) lv->dx[d] = tmp_dx[cl + i - 1][d];
      for (b = 0; b < lv->nbox; b++) {
         h->boxes[lv->box[b]].level = i;
         if (i == 1) h->boxes[lv->box[b]].coarsest = 1;
      }
   }
   for (l = prm->min_level; l <= h->n_amr; l++) free(amr_list[l]);
   /* AMR-level boxes keep coarsest = 0 except on MG level 1 (gh.c:1137, 1357) */
   for (i = 0; i < h->nbox; i++) {
      pgb_hbox *b = &h->boxes[i];
      int pow2 = 1, iso = 1;
      double dx0 = b->x[0][1] - b->x[0][0];
      if (b->level != 1 && b->amr_grid >= 0) b->coarsest = 0;
      for (d = 0; d < dim; d++) {
         double dxo = b->x[d][1] - b->x[d][0];
         if (!is_pow2(dxo * dxo)) pow2 = 0;
         if (dxo * dxo != dx0 * dx0) iso = 0;
      }
      if (pow2) b->flags |= PGB_BOX_POW2DX;
      if (iso) b->flags |= PGB_BOX_ISO;
      if (b->coarsest) b->flags |= PGB_BOX_COARSEST;
   }
   build_masks(h);

   /* transfer bits for this variable set (PAMR_set_tf_bits src/pamr.c:1826-1878,
      variable attributes amrd/io.c:743-871) */
   memset(ops_init, 0, sizeof(ops_init));
   memset(ops_inj, 0, sizeof(ops_inj));
   memset(ops_inj_mg, 0, sizeof(ops_inj_mg));
   memset(ops_sync, 0, sizeof(ops_sync));
   memset(ops_int, 0, sizeof(ops_int));
   for (i = 0; i < (prm->nsrc > 1 ? prm->nsrc : 1); i++) {
      const int op = i ? prm->restr_srck[i] : prm->restr_src;
      ops_init[PGB_SRC_FIELD(i)] = op;      /* in both hierarchies, mg_inject set */
      ops_inj_mg[PGB_SRC_FIELD(i)] = op;    /* sources have mg_noinj_to_amr = 1 */
   }
   for (i = 0; i < (prm->nvar > 1 ? prm->nvar : 1); i++) {   /* every elliptic variable alike */
      ops_init[PGB_FV(i, PGB_F_U)] = prm->restr_u;
      ops_inj[PGB_FV(i, PGB_F_U)] = prm->restr_u;
      ops_inj[PGB_FV(i, PGB_F_RES)] = prm->restr_res;
      ops_inj_mg[PGB_FV(i, PGB_F_U)] = prm->restr_u;
      ops_inj_mg[PGB_FV(i, PGB_F_RES)] = prm->restr_res;
      ops_sync[PGB_FV(i, PGB_F_U)] = 1;
      ops_int[PGB_FV(i, PGB_F_RES)] = prm->interp_order;
   }
   (void)ops_sync;
   for (l = 1; l <= nl; l++) {
      plan_comm(h, COMM_SYNC, l, l, 1, 0, 0, 0, &h->sync[l][0]);
      plan_comm(h, COMM_SYNC, l, l, 2, 0, 0, 0, &h->sync[l][1]);
      plan_comm(h, COMM_SYNC, l, l, 2, 0, 1, 0, &h->sync_coarsest[l]);
      if (l < nl) {
         plan_comm(h, COMM_INJECT, l + 1, l, 1, 0, 0, h->lev[l].in_amrh ? ops_inj : ops_inj_mg,
                   &h->inject[l]);
         if (!h->lev[l].in_amrh) plan_comm(h, COMM_INJECT, l + 1, l, 1, 0, 0, ops_init, &h->inject_init[l]);
      }
      if (l > 1) plan_comm(h, COMM_INTERP, l - 1, l, 0, 1, 0, ops_int, &h->interp[l]);
   }
   if (h->err[0]) return 2;
   return 0;
}

/* MG level of AMR level L (the L-th level kept in the AMR hierarchy), 0 if none */
static int amr_level_to_mg(const pgb_hier *h, int L)
{
   int l, k = 0;
   for (l = 1; l <= h->nlev; l++)
      if (h->lev[l].in_amrh && ++k == L - h->prm.min_level + 1) return l;
   return 0;
}

int pgb_plan_amr_interp(pgb_hier *h, int lc, int amr_bdy_width, int order, pgb_plan *out)
{
   int ops[PGB_NF], f;
   const int mc = amr_level_to_mg(h, lc), mf = amr_level_to_mg(h, lc + 1);
   memset(out, 0, sizeof(*out));
   if (!mc || !mf) {
      snprintf(h->err, sizeof(h->err), "AMR levels %d and %d are not both in the hierarchy", lc, lc + 1);
      return 1;
   }
   for (f = 0; f < PGB_NF; f++) ops[f] = order;
   h->err[0] = 0;
   plan_comm_bdy(h, COMM_INTERP, mc, mf, 0, 1, 0, amr_bdy_width, ops, out);
   return h->err[0] ? 2 : 0;
}

/* init_new_cgh (src/gh.c:934-1045) for AMR level Ln of the hierarchy hn
 * built after a regrid, from the hierarchy ho it replaces: with interp set,
 * the interpolation of order `order` from ho's level Ln-1 (owned, extended
 * by one point: build_owned_gsl(.., 0, 1)) into every grid of hn's level Ln
 * (build_complete_gsl), then the copies from ho's level Ln (owned) into
 * hn's level Ln where the grids overlap. The two transfers run through the
 * same gsl algebra and op lists as PAMR_interp and PAMR_sync, on a joint box
 * list: ho's boxes first, then hn's (box index + ho->nbox). A level missing
 * from ho gives an empty plan. Returns 0, or 1 with err filled. */
int pgb_plan_regrid(const pgb_hier *ho, const pgb_hier *hn, int Ln, int order, int interp, pgb_plan *pi,
                    pgb_plan *pc, char *err, size_t errlen)
{
   pgb_hier t;
   int ops[PGB_NF], f, b, rc = 0;
   const int mo1 = Ln - 1 >= ho->prm.min_level ? amr_level_to_mg(ho, Ln - 1) : 0;
   const int mo = amr_level_to_mg(ho, Ln), mn = amr_level_to_mg(hn, Ln);
   memset(pi, 0, sizeof(*pi));
   memset(pc, 0, sizeof(*pc));
   if (!mn) {
      snprintf(err, errlen, "AMR level %d is not in the new hierarchy", Ln);
      return 1;
   }
   memset(&t, 0, sizeof(t));
   t.dim = hn->dim;
   t.pde = hn->pde;
   memcpy(t.base_shape, hn->base_shape, sizeof(t.base_shape));
   memcpy(t.base_bbox, hn->base_bbox, sizeof(t.base_bbox));
   t.prm = hn->prm;
   t.nbox = ho->nbox + hn->nbox;
   t.boxes = (pgb_hbox *)malloc(sizeof(pgb_hbox) * (size_t)t.nbox);   /* shallow: masks and x stay theirs */
   memcpy(t.boxes, ho->boxes, sizeof(pgb_hbox) * (size_t)ho->nbox);
   memcpy(t.boxes + ho->nbox, hn->boxes, sizeof(pgb_hbox) * (size_t)hn->nbox);
   t.nlev = 3;
   if (mo1) t.lev[1] = ho->lev[mo1];
   if (mo) t.lev[2] = ho->lev[mo];
   t.lev[3] = hn->lev[mn];
   t.lev[3].box = (int *)malloc(sizeof(int) * (size_t)(hn->lev[mn].nbox + 1));
   for (b = 0; b < hn->lev[mn].nbox; b++) t.lev[3].box[b] = hn->lev[mn].box[b] + ho->nbox;
   for (f = 0; f < PGB_NF; f++) ops[f] = order;
   if (interp && mo1) plan_comm(&t, COMM_INTERP, 1, 3, 0, 1, 0, ops, pi);
   if (!t.err[0] && mo) plan_comm(&t, COMM_SYNC, 2, 3, 0, 0, 0, 0, pc);
   if (t.err[0]) {
      snprintf(err, errlen, "%s", t.err);
      rc = 1;
   }
   free(t.lev[3].box);
   free(t.boxes);
   return rc;
}

void pgb_plan_release(pgb_plan *p)
{
   free(p->batch_start);
   free(p->batch_maxpts);
   free(p->h_ops);
   memset(p, 0, sizeof(*p));
}

static void plan_free(pgb_plan *p)
{
   free(p->batch_start);
   free(p->batch_maxpts);
   free(p->h_ops);
   memset(p, 0, sizeof(*p));
}

void pgb_hier_free(pgb_hier *h)
{
   int i, d, l;
   for (i = 0; i < h->nbox; i++) {
      for (d = 0; d < 3; d++) free(h->boxes[i].x[d]);
      free(h->boxes[i].child_mask);
      free(h->boxes[i].bdy_mask);
   }
   free(h->boxes);
   free(h->grid_box);
   for (l = 1; l <= h->nlev; l++) {
      free(h->lev[l].box);
      plan_free(&h->sync[l][0]);
      plan_free(&h->sync[l][1]);
      plan_free(&h->sync_coarsest[l]);
      plan_free(&h->inject[l]);
      plan_free(&h->inject_init[l]);
      plan_free(&h->interp[l]);
   }
   memset(h, 0, sizeof(*h));
}
