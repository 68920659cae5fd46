/*
 * libpamr_gb300 host driver (C): device arena, plan upload and the FAS
 * V-cycle of amrd/mg.c:84-201 issued as kernel launches on one stream.
 *
 * The control flow is the reference's; every norm stays on the device (the
 * coarsest-grid loop runs inside one kernel), so a V-cycle needs a single
 * device-to-host read: the finest residual that solve_elliptics compares
 * with MG_tol (amrd/mg.c:57).
 */
#include <cuda_runtime_api.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "pamr_gb300.h"
#include "pgb_dev.h"
#include "pgb_plan.h"

/* norm slots per level */
enum { N_RELAX_DN = 0, N_RELAX_UP = 1, N_RESID = 2, N_COARSE = 3, N_SLOTS = 4 };

struct pgb_solver {
   pgb_hier h;
   pgb_dop dop;             /* the level operator (kind also in h.pde) */
   pgb_dop *d_dop;          /* device copies of the variables' operators, which every box points to */
   int nsrc;                /* source fields allocated per box (>= 1) */
   int nvar;                /* elliptic variables (AMRD_num_elliptic_vars) */
   pgb_dop dops[PGB_NVAR_MAX]; /* operator of each variable (dops[0] = dop) */
   int host_only;
   cudaStream_t stream;
   char *arena;
   size_t arena_bytes;
   pgb_dbox *hbox;          /* host copy of the device box table */
   pgb_dbox *dbox;
   /* mixed form with several elliptic variables: the box table as the
    * one-variable kernels see variable v (vbox[0] = dbox): its U..RHS fields
    * and variable 0's swapped, its own FP32 arrays, its operator renumbered
    * to match (d_vdop[v]) */
   pgb_dbox *vbox[PGB_NVAR_MAX];
   pgb_dop *d_vdop;
   pgb_dlevel lv[PGB_MAXLEV + 1];
   void *d_tables[PGB_MAXLEV + 1];
   pgb_scratch sc;
   double *d_norms;         /* [(nlev+1) * N_SLOTS] */
   int *d_citers;
   double *d_snap;
   long snap_points;
   long *d_snap_off[PGB_MAXLEV + 1];
   pgb_trace *d_trace;
   int trace_cap;
   double *h_res;           /* pinned */
   int prepared;            /* pgb_prepare ran after the last change of an input grid */
   int fuse[PGB_MAXLEV + 1]; /* mixed form: FP32 sweeps per launch on levels without syncs */
   int eslot[PGB_MAXLEV + 1]; /* mixed form: slot of E = 0 after a level's pre-smoothing block */
   int res32[PGB_MAXLEV + 1]; /* mixed form: level's residual restricted from its FP32 copy */
   int tuned;               /* the autotuner has run */
   int dnext[PGB_MAXLEV + 1]; /* mixed form: pre-smoothing defect from the FP32 update (see
                               k_defect32) outside the cover tiles */
   cudaGraphExec_t gexec;   /* one captured V-cycle (+ read-back of the residual) */
   int graph_ok;
   long long graph_kernels; /* kernel launches in the captured V-cycle */
   cudaGraphExec_t sexec;   /* the solve loop: V-cycles under a conditional while node */
   int solve_ok;            /* 1 built, -1 not available (host loop) */
   cudaGraphExec_t pexec;   /* pgb_prepare's launches (after the autotuner ran), replayed by pgb_solve */
   int prep_ok;             /* 1 built, -1 not available */
   double *d_hist;          /* finest residual after each cycle of a solve [max_iter] */
   int *d_parity;           /* mixed form: 0 / 1 for even / odd cycles of a solve */
   void *d_tmaps;           /* mixed form, 3-D: tensor maps of the TMA-staged sweep (0: unavailable) */
   int *d_err;              /* set by a device wait that timed out */
   int mtx[PGB_MAXLEV + 1]; /* output width of the TMA sweep's columns per level (60 or 28) */
   int mtz[PGB_MAXLEV + 1]; /* planes per column of the TMA sweep per level (4 to 64; even) */
   int *d_it;               /* cycles run by the device loop */
   cudaEvent_t ev0, ev1;
   cudaStream_t side;       /* second stream for independent kernels of a cycle */
   cudaEvent_t evfork, evjoin;
   int last_cycles;
   long last_citers;
   double last_ms;
   int tail_lc;             /* mixed form: levels 1..tail_lc run in the small-level kernel (0: none) */
   int tail_ncta;           /* its cluster size */
   int tail_solo;           /* levels 1..tail_solo of those run in one CTA (their steps need no cluster) */
   int tail_grid;           /* 0: one cluster; else the CTAs of a cooperative launch (one per SM) */
   size_t tail_mini;        /* mini mode: bytes of the levels' arrays staged in one CTA's shared memory */
   unsigned int *d_tailbar; /* its barrier counter */
   pgb_tail_prog *tail;     /* its program, recorded by each V-cycle launch or capture */
};

static __thread char g_err[512];
static long long g_graph_replayed = 0, g_captured = 0;

const char *pgb_last_error(void) { return g_err; }

/* lets the device entry points that take no solver (pgb_dm*) report too */
void pgb_note_error(const char *msg) { snprintf(g_err, sizeof(g_err), "%s", msg); }

static int fail(int code, const char *fmt, ...)
{
   va_list ap;
   va_start(ap, fmt);
   vsnprintf(g_err, sizeof(g_err), fmt, ap);
   va_end(ap);
   return code;
}

#define CU(call)                                                                    \
   do {                                                                             \
      cudaError_t e_ = (call);                                                      \
      if (e_ != cudaSuccess) return fail(10, "%s: %s", #call, cudaGetErrorString(e_)); \
   } while (0)
#define KC(call)                                                                    \
   do {                                                                             \
      if (call) return fail(11, "%s", pgb_dev_error());                              \
   } while (0)
#define KC32(call)                                                                  \
   do {                                                                             \
      if (call) return fail(11, "%s", pgb_dev_error32());                            \
   } while (0)

static void drop_graph(pgb_solver *s);

void pgb_default_params(pgb_mg_params *p)
{
   memset(p, 0, sizeof(*p));
   p->pre_swp = p->pst_swp = 2;
   p->max_iter = 50;
   p->min_iter = 1;
   p->max_citer = 5000;
   p->tol = 0;
   p->crtol = 1.0e-3;
   p->w0_r = p->w0_i = 1.0;
   p->min_cwidth = 3;
   p->restr_u = PGB_HW_RESTR;
   p->restr_res = PGB_FW_RESTR;
   p->restr_src = PGB_HW_RESTR;
   p->interp_order = 2;
   p->interp_buffer = 2;
   p->precision = PGB_FP64;
}

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

/* planes per tile: the largest of 8, 4, 2, 1 that still gives the level at
 * least two CTAs per SM of GB300 (152 SMs) */
static int choose_tz(const pgb_hier *h, int L, int tx)
{
   int tz, b;
   if (h->dim != 3) return 1;
   for (tz = PGB_TZ; tz > 1; tz /= 2) {
      long n = 0;
      for (b = 0; b < h->lev[L].nbox; b++) {
         const pgb_hbox *bx = &h->boxes[h->lev[L].box[b]];
         n += (long)((bx->shape[0] + tx - 1) / tx) * ((bx->shape[1] + PGB_TY - 1) / PGB_TY) *
              ((bx->shape[2] + tz - 1) / tz);
      }
      if (n >= 2 * 152) break;
   }
   return tz;
}

/* The subset of a level's tiles that the coarse half of the coarse-grid
 * correction and the FAS right-hand side have to visit: tiles that contain a
 * point with the child cmask ON, or a point inside the coarse window of an
 * interpolation op to level L+1. Elsewhere rhs stays 0 (cleared by
 * pgb_prepare, never written by a cycle) and lop/res are never read before
 * the next clear or residual, so skipping those tiles changes no result. */
static int make_cover_tiles(const pgb_hier *h, int L, const pgb_tile *t, int nt, int tz,
                            pgb_tile **out)
{
   int n = 0, q;
   pgb_tile *c = (pgb_tile *)malloc(sizeof(pgb_tile) * (size_t)(nt ? nt : 1));
   const pgb_plan *ip = L < h->nlev ? &h->interp[L + 1] : 0;
   for (q = 0; q < nt; q++) {
      const pgb_hbox *bx = &h->boxes[t[q].box];
      int lo[3] = {t[q].i0, t[q].j0, t[q].k0};
      int hi[3] = {t[q].i0 + PGB_TX - 1, t[q].j0 + PGB_TY - 1, h->dim == 3 ? t[q].k0 + tz - 1 : 0};
      int d, i, j, k, hit = 0;
      for (d = 0; d < 3; d++)
         if (hi[d] > bx->shape[d] - 1) hi[d] = bx->shape[d] - 1;
      for (k = lo[2]; k <= hi[2] && !hit; k++)
         for (j = lo[1]; j <= hi[1] && !hit; j++)
            for (i = lo[0]; i <= hi[0]; i++)
               if (bx->child_mask[i + (long)bx->shape[0] * (j + (long)bx->shape[1] * k)]) {
                  hit = 1;
                  break;
               }
      if (!hit && ip) {
         const pgb_interp_op *o = (const pgb_interp_op *)ip->h_ops;
         int m;
         for (m = 0; m < ip->nops && !hit; m++) {
            int wlo[3] = {o[m].i1i - 1, o[m].j1i - 1, o[m].k1i - 1};
            int whi[3] = {wlo[0] + o[m].nii - 1, wlo[1] + o[m].nji - 1, wlo[2] + o[m].nki - 1};
            if (o[m].src_box != t[q].box) continue;
            hit = 1;
            for (d = 0; d < h->dim; d++)
               if (whi[d] < lo[d] || wlo[d] > hi[d]) hit = 0;
         }
      }
      if (hit) c[n++] = t[q];
   }
   *out = c;
   return n;
}

/* tiles of the boxes of one level; tx = tile width in x, tz planes deep */
static int make_tiles(const pgb_hier *h, int L, int tx, int tz, pgb_tile **out, int *start)
{
   int b, n = 0, cap = 64;
   pgb_tile *t = (pgb_tile *)malloc(sizeof(pgb_tile) * (size_t)cap);
   for (b = 0; b < h->lev[L].nbox; b++) {
      const pgb_hbox *bx = &h->boxes[h->lev[L].box[b]];
      int i, j, k;
      start[b] = n;
      for (k = 0; k < bx->shape[2]; k += tz)
         for (j = 0; j < bx->shape[1]; j += PGB_TY)
            for (i = 0; i < bx->shape[0]; i += tx) {
               if (n == cap) {
                  cap *= 2;
                  t = (pgb_tile *)realloc(t, sizeof(pgb_tile) * (size_t)cap);
               }
               t[n].box = h->lev[L].box[b];
               t[n].i0 = i;
               t[n].j0 = j;
               t[n].k0 = k;
               t[n].slot = n;
               n++;
            }
   }
   start[h->lev[L].nbox] = n;
   *out = t;
   return n;
}

/* tiles of tx x ty x tz points over the boxes of one level */
static int make_tiles2(const pgb_hier *h, int L, int tx, int ty, int tz, pgb_tile **out, int *start)
{
   int b, n = 0, cap = 64;
   pgb_tile *t = (pgb_tile *)malloc(sizeof(pgb_tile) * (size_t)cap);
   for (b = 0; b < h->lev[L].nbox; b++) {
      const pgb_hbox *bx = &h->boxes[h->lev[L].box[b]];
      int i, j, k;
      start[b] = n;
      for (k = 0; k < bx->shape[2]; k += tz)
         for (j = 0; j < bx->shape[1]; j += ty)
            for (i = 0; i < bx->shape[0]; i += tx) {
               if (n == cap) {
                  cap *= 2;
                  t = (pgb_tile *)realloc(t, sizeof(pgb_tile) * (size_t)cap);
               }
               t[n].box = h->lev[L].box[b];
               t[n].i0 = i;
               t[n].j0 = j;
               t[n].k0 = k;
               t[n].slot = n;
               n++;
            }
   }
   start[h->lev[L].nbox] = n;
   *out = t;
   return n;
}

/* the TMA-staged sweep needs tensor maps and boxes whose interior is all relaxed */
static int level_tma_ok(const pgb_solver *s, int L)
{
   int b;
   if (!s->d_tmaps || s->h.dim != 3) return 0;
   for (b = 0; b < s->h.lev[L].nbox; b++)
      if (!(s->h.boxes[s->h.lev[L].box[b]].flags & PGB_BOX_BDY_INTERIOR)) return 0;
   return 1;
}

static int upload_plan(pgb_plan *p, size_t opsz)
{
   if (!p->nops) return 0;
   CU(cudaMalloc(&p->d_ops, opsz * (size_t)p->nops));
   CU(cudaMemcpy(p->d_ops, p->h_ops, opsz * (size_t)p->nops, cudaMemcpyHostToDevice));
   return 0;
}

static void free_plan_dev(pgb_plan *p)
{
   if (p->d_ops) cudaFree(p->d_ops);
   p->d_ops = 0;
}

/* (Re)builds the device tables of level L: tiles of tz planes, relax tiles,
 * tile starts, the box list and the cover tiles. */
static int level_tables(pgb_solver *s, int L, int tz)
{
   pgb_hier *h = &s->h;
   pgb_tile *t = 0, *rt = 0, *ct = 0, *zt = 0;
   int nb = h->lev[L].nbox, nct;
   int *ts = (int *)malloc(sizeof(int) * (size_t)(nb + 1));
   int *rts = (int *)malloc(sizeof(int) * (size_t)(nb + 1));
   int *zts = (int *)malloc(sizeof(int) * (size_t)(nb + 1));
   int rtz = tz, ztz = h->dim == 3 ? 4 * tz : 1;
   const int mtx = s->mtx[L] ? s->mtx[L] : 60, mtz = s->mtz[L] ? s->mtz[L] : 32;
   pgb_tile *mt = 0;
   int *mts = (int *)malloc(sizeof(int) * (size_t)(nb + 1));
   int nt = make_tiles(h, L, PGB_TX, tz, &t, ts);
   int nrt = make_tiles(h, L, 2 * PGB_TX, rtz, &rt, rts);
   int nzt = make_tiles(h, L, PGB_TX, ztz, &zt, zts);
   int nmt = h->dim == 3 ? make_tiles2(h, L, mtx, 14, mtz, &mt, mts) : 0;
   size_t b0 = 0, b1 = align256(sizeof(pgb_tile) * (size_t)nt);
   size_t b2 = b1 + align256(sizeof(pgb_tile) * (size_t)nrt);
   size_t b3 = b2 + align256(sizeof(int) * (size_t)(nb + 1));
   size_t b4 = b3 + align256(sizeof(int) * (size_t)(nb + 1));
   size_t b5 = b4 + align256(sizeof(int) * (size_t)nb), b6;
   char *dt;
   int rc = 0;
   nct = make_cover_tiles(h, L, t, nt, tz, &ct);
   b6 = b5 + align256(sizeof(pgb_tile) * (size_t)(nct ? nct : 1));
   size_t b7 = b6 + align256(sizeof(pgb_tile) * (size_t)nzt);
   size_t b8 = b7 + align256(sizeof(pgb_tile) * (size_t)(nmt ? nmt : 1));
   if (s->d_tables[L]) cudaFree(s->d_tables[L]);
   s->d_tables[L] = 0;
   if (cudaMalloc(&s->d_tables[L], b8) != cudaSuccess) {
      rc = fail(10, "cudaMalloc of the level tables failed");
      goto out;
   }
   dt = (char *)s->d_tables[L];
   if ((nct && cudaMemcpy(dt + b5, ct, sizeof(pgb_tile) * (size_t)nct, cudaMemcpyHostToDevice)) ||
       cudaMemcpy(dt + b0, t, sizeof(pgb_tile) * (size_t)nt, cudaMemcpyHostToDevice) ||
       cudaMemcpy(dt + b1, rt, sizeof(pgb_tile) * (size_t)nrt, cudaMemcpyHostToDevice) ||
       cudaMemcpy(dt + b2, ts, sizeof(int) * (size_t)(nb + 1), cudaMemcpyHostToDevice) ||
       cudaMemcpy(dt + b3, rts, sizeof(int) * (size_t)(nb + 1), cudaMemcpyHostToDevice) ||
       cudaMemcpy(dt + b4, h->lev[L].box, sizeof(int) * (size_t)nb, cudaMemcpyHostToDevice) ||
       cudaMemcpy(dt + b6, zt, sizeof(pgb_tile) * (size_t)nzt, cudaMemcpyHostToDevice) ||
       (nmt && cudaMemcpy(dt + b7, mt, sizeof(pgb_tile) * (size_t)nmt, cudaMemcpyHostToDevice))) {
      rc = fail(10, "upload of the level tables failed");
      goto out;
   }
   s->lv[L].tiles = (const pgb_tile *)(dt + b0);
   s->lv[L].rtiles = (const pgb_tile *)(dt + b1);
   s->lv[L].tile_start = (const int *)(dt + b2);
   s->lv[L].rtile_start = (const int *)(dt + b3);
   s->lv[L].box = (const int *)(dt + b4);
   s->lv[L].ctiles = (const pgb_tile *)(dt + b5);
   s->lv[L].nctiles = nct;
   s->lv[L].ztiles = (const pgb_tile *)(dt + b6);
   s->lv[L].nztiles = nzt;
   s->lv[L].ztz = ztz;
   s->lv[L].mtiles = (const pgb_tile *)(dt + b7);
   s->lv[L].nmtiles = nmt;
   s->lv[L].mtx = mtx;
   s->lv[L].mtz = mtz;
   s->lv[L].tmaps = level_tma_ok(s, L) ? s->d_tmaps : 0;
   s->lv[L].err = s->d_err;
   s->lv[L].ntiles = nt;
   s->lv[L].nrtiles = nrt;
   s->lv[L].nbox = nb;
   s->lv[L].tz = tz;
   s->lv[L].rtz = rtz;
   s->lv[L].dim = h->dim;
   s->lv[L].level = L;
   s->lv[L].nvar = s->nvar;
out:
   free(t);
   free(rt);
   free(ct);
   free(zt);
   free(ts);
   free(rts);
   free(zts);
   free(mt);
   free(mts);
   return rc;
}

/* grid functions a box of this solver carries: variable 0's and those of
 * its other elliptic variables, the sources its operators read */
static int field_used(const pgb_solver *s, int f)
{
   if (f >= PGB_F_VAR1) return 1 + (f - PGB_F_VAR1) / 4 < s->nvar;
   if (f >= PGB_F_SRC1) return f - PGB_F_SRC1 + 1 < s->nsrc;
   return 1;
}

/* The views of a mixed-form solver with several elliptic variables. The
 * FP32 passes (sweeps, defect, update, coarse-grid correction,
 * interpolation) and the FP64 passes of one variable (residual, FAS
 * right-hand side) are one-variable kernels: run over the box table of view
 * v, they read and write variable v. View v swaps the U, RES, LOP and RHS
 * slots of variables 0 and v, points the FP32 arrays (and the coupling
 * coefficients) at variable v's, and
 * gives the boxes variable v's operator with its variable names renumbered
 * by the same swap, so that the other variables it names are read from the
 * slots that hold them (pgb_prog_vars, pgb_op.cuh). View 0 is the box table
 * itself. */
static int var_views(pgb_solver *s, const size_t *w32o, int per)
{
   const int nw32 = per * s->nvar;
   const pgb_hier *h = &s->h;
   pgb_dop vd[PGB_NVAR_MAX];
   pgb_dbox *t;
   int v, i, f, q, rc = 0;
   for (v = 0; v < s->nvar; v++) {
      vd[v] = s->dops[v];
      for (q = 0; q < 2; q++) {
         unsigned char *code = q ? vd[v].jcode : vd[v].lcode;
         for (i = 0; i < PGB_PROG_MAX && (code[i] & 15) != PGB_P_END; i++) {
            const int a = code[i] >> 4;
            if ((code[i] & 15) == PGB_P_U && a >= 1) {   /* u<a-1>: variable a-1 sits in slot swap(a-1) */
               const int k = a - 1, sk = k == 0 ? v : k == v ? 0 : k;
               code[i] = (unsigned char)(((sk + 1) << 4) | PGB_P_U);
            }
         }
      }
   }
   CU(cudaMalloc((void **)&s->d_vdop, sizeof(pgb_dop) * (size_t)s->nvar));
   CU(cudaMemcpy(s->d_vdop, vd, sizeof(pgb_dop) * (size_t)s->nvar, cudaMemcpyHostToDevice));
   t = (pgb_dbox *)malloc(sizeof(pgb_dbox) * (size_t)h->nbox);
   if (!t) return fail(10, "out of host memory");
   for (v = 1; v < s->nvar && !rc; v++) {
      for (i = 0; i < h->nbox; i++) {
         t[i] = s->hbox[i];
         for (f = PGB_F_U; f <= PGB_F_RHS; f++) {
            t[i].f[f] = s->hbox[i].f[PGB_FV(v, f)];
            t[i].f[PGB_FV(v, f)] = s->hbox[i].f[f];
         }
         for (f = 0; f < PGB_NW32; f++) t[i].w32[f] = (float *)(s->arena + w32o[i * nw32 + v * per + f]);
         t[i].w32c = (float *)(s->arena + w32o[i * nw32 + v * per + PGB_NW32]);
         t[i].op = s->d_vdop + v;
      }
      if (cudaMalloc((void **)&s->vbox[v], sizeof(pgb_dbox) * (size_t)h->nbox) != cudaSuccess ||
          cudaMemcpy(s->vbox[v], t, sizeof(pgb_dbox) * (size_t)h->nbox, cudaMemcpyHostToDevice) != cudaSuccess)
         rc = fail(10, "variable views: out of device memory");
   }
   free(t);
   return rc;
}

static int setup_device(pgb_solver *s)
{
   pgb_hier *h = &s->h;
   size_t off = 0, *fo, *w32o = 0;
   int i, f, L, d, rc, maxt = 1, maxbox = 1;
   /* mixed form: per box and variable PGB_NW32 FP32 arrays, and with several
    * variables one block of nvar - 1 arrays of coupling coefficients */
   const int per = PGB_NW32 + (s->nvar > 1), nw32 = per * s->nvar;
   long snap_pts = 0;
   {
      /* the solver's streams at the device's greatest priority: a V-cycle
       * is a chain of short dependent kernels, and work another stream runs
       * beside it (the next solve's learned guess) should take the SMs its
       * kernels leave free, not delay them (PGB_NO_STREAM_PRIORITY=1: the
       * default priority) */
      int least = 0, greatest = 0;
      if (getenv("PGB_NO_STREAM_PRIORITY") || cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess)
         greatest = 0;
      CU(cudaStreamCreateWithPriority(&s->stream, cudaStreamNonBlocking, greatest));
      CU(cudaStreamCreateWithPriority(&s->side, cudaStreamNonBlocking, greatest));
   }
   CU(cudaEventCreate(&s->ev0));
   CU(cudaEventCreate(&s->ev1));
   CU(cudaEventCreateWithFlags(&s->evfork, cudaEventDisableTiming));
   CU(cudaEventCreateWithFlags(&s->evjoin, cudaEventDisableTiming));
   /* arena layout: per box, 5 float64 grid functions then 2 byte masks */
   fo = (size_t *)malloc(sizeof(size_t) * (size_t)h->nbox * (PGB_NF + 2));
   for (i = 0; i < h->nbox; i++) {
      const pgb_hbox *b = &h->boxes[i];
      size_t n = (size_t)b->shape[0] * b->shape[1] * b->shape[2];
      for (f = 0; f < PGB_NF; f++) {
         fo[i * (PGB_NF + 2) + f] = off;
         if (!field_used(s, f)) continue;   /* source the operator does not read, variable it lacks */
         off = align256(off + 8 * n);
      }
      fo[i * (PGB_NF + 2) + PGB_NF] = off;
      off = align256(off + n);
      fo[i * (PGB_NF + 2) + PGB_NF + 1] = off;
      off = align256(off + n);
   }
   if (h->prm.precision == PGB_MIXED) {
      w32o = (size_t *)malloc(sizeof(size_t) * (size_t)h->nbox * nw32);
      for (i = 0; i < h->nbox; i++) {
         const pgb_hbox *b = &h->boxes[i];
         /* rows padded to a multiple of 4 floats (16 bytes) */
         size_t n = (size_t)((b->shape[0] + 3) & ~3) * b->shape[1] * b->shape[2];
         for (f = 0; f < nw32; f++) {
            w32o[i * nw32 + f] = off;
            off = align256(off + 4 * n * (f % per == PGB_NW32 ? (size_t)(s->nvar - 1) : 1));
         }
      }
   }
   s->arena_bytes = off;
   CU(cudaMalloc((void **)&s->d_dop, sizeof(pgb_dop) * (size_t)s->nvar));
   CU(cudaMemcpy(s->d_dop, s->dops, sizeof(pgb_dop) * (size_t)s->nvar, cudaMemcpyHostToDevice));
   CU(cudaMalloc((void **)&s->arena, off));
   CU(cudaMemset(s->arena, 0, off));
   s->hbox = (pgb_dbox *)calloc((size_t)h->nbox, sizeof(pgb_dbox));
   for (i = 0; i < h->nbox; i++) {
      const pgb_hbox *b = &h->boxes[i];
      pgb_dbox *db = &s->hbox[i];
      size_t n = (size_t)b->shape[0] * b->shape[1] * b->shape[2];
      double dx2[3] = {1, 1, 1};
      for (f = 0; f < PGB_NF; f++) db->f[f] = field_used(s, f) ? (double *)(s->arena + fo[i * (PGB_NF + 2) + f]) : 0;
      db->op = s->d_dop;
      if (w32o)
         for (f = 0; f < PGB_NW32; f++) db->w32[f] = (float *)(s->arena + w32o[i * nw32 + f]);
      if (w32o && s->nvar > 1) db->w32c = (float *)(s->arena + w32o[i * nw32 + PGB_NW32]);
      db->cmask_child = (const uint8_t *)(s->arena + fo[i * (PGB_NF + 2) + PGB_NF]);
      db->cmask_bdy = (const uint8_t *)(s->arena + fo[i * (PGB_NF + 2) + PGB_NF + 1]);
      CU(cudaMemcpy((void *)db->cmask_child, b->child_mask, n, cudaMemcpyHostToDevice));
      CU(cudaMemcpy((void *)db->cmask_bdy, b->bdy_mask, n, cudaMemcpyHostToDevice));
      for (d = 0; d < 3; d++) db->n[d] = b->shape[d];
      db->wy = (b->shape[0] + 3) & ~3;
      db->wz = (long)db->wy * b->shape[1];
      db->flags = b->flags;
      db->level = b->level;
      db->count = b->count;
      /* dx = x(2)-x(1) of the grid's coordinates, dx2 = dx**2 (num.f:191-197) */
      for (d = 0; d < h->dim; d++) {
         double dx = b->x[d][1] - b->x[d][0];
         dx2[d] = dx * dx;
      }
      for (d = 0; d < 3; d++) {
         db->dx2[d] = dx2[d];
         db->idx2[d] = 1.0 / dx2[d];
      }
      if (h->dim == 3) db->j0 = -2 / dx2[0] - 2 / dx2[1] - 2 / dx2[2];
      else db->j0 = -2 / dx2[0] - 2 / dx2[1];
      for (d = 0; d < 3; d++) db->fidx2[d] = (float)db->idx2[d];
      db->fj0 = (float)db->j0;
   }
   free(fo);
   CU(cudaMalloc((void **)&s->dbox, sizeof(pgb_dbox) * (size_t)h->nbox));
   CU(cudaMemcpy(s->dbox, s->hbox, sizeof(pgb_dbox) * (size_t)h->nbox, cudaMemcpyHostToDevice));
   s->vbox[0] = s->dbox;
   rc = w32o && s->nvar > 1 ? var_views(s, w32o, per) : 0;
   free(w32o);
   if (rc) return rc;
   CU(cudaMalloc((void **)&s->d_err, sizeof(int)));
   CU(cudaMemset(s->d_err, 0, sizeof(int)));
   if (h->prm.precision == PGB_MIXED && h->dim == 3 && s->nvar == 1 && !getenv("PGB_NO_TMA"))
      pgb_tmaps_build(s->hbox, h->nbox, &s->d_tmaps);   /* 1 (no maps): the TMA sweep is not offered */

   /* per-level tables: tiles, relax tiles, tile starts, box lists */
   for (L = 1; L <= h->nlev; L++) {
      int nb = h->lev[L].nbox;
      if (level_tables(s, L, choose_tz(h, L, PGB_TX))) return 10;
      s->fuse[L] = 0;
      /* the reduction scratch holds the partial sums of the most finely
       * tiled layout the autotuner can pick (one plane per tile) */
      {
         long n1 = 0;
         int b;
         for (b = 0; b < nb; b++) {
            const pgb_hbox *bx = &h->boxes[h->lev[L].box[b]];
            n1 += (long)((bx->shape[0] + PGB_TX - 1) / PGB_TX) * ((bx->shape[1] + PGB_TY - 1) / PGB_TY) *
                  bx->shape[2];
         }
         if (n1 > maxt) maxt = (int)n1;
         if (s->lv[L].nrtiles > maxt) maxt = s->lv[L].nrtiles;
      }
      if (nb > maxbox) maxbox = nb;
      /* snapshot offsets of the coarsest boxes of this level */
      {
         long o = 0, *so = (long *)calloc((size_t)nb + 1, sizeof(long));
         int any = 0;
         for (i = 0; i < nb; i++) {
            const pgb_hbox *b = &h->boxes[h->lev[L].box[i]];
            so[i] = o;
            if (b->coarsest) {
               o += (long)b->shape[0] * b->shape[1] * b->shape[2];
               any = 1;
            }
         }
         so[nb] = o;
         if (any) {
            CU(cudaMalloc((void **)&s->d_snap_off[L], sizeof(long) * (size_t)(nb + 1)));
            CU(cudaMemcpy(s->d_snap_off[L], so, sizeof(long) * (size_t)(nb + 1), cudaMemcpyHostToDevice));
         }
         if (o > snap_pts) snap_pts = o;
         free(so);
      }
      if (upload_plan(&h->sync[L][0], sizeof(pgb_copy_op)) ||
          upload_plan(&h->sync[L][1], sizeof(pgb_copy_op)) ||
          upload_plan(&h->sync_coarsest[L], sizeof(pgb_copy_op)) ||
          upload_plan(&h->inject[L], sizeof(pgb_restrict_op)) ||
          upload_plan(&h->inject_init[L], sizeof(pgb_restrict_op)) ||
          upload_plan(&h->interp[L], sizeof(pgb_interp_op)))
         return 10;
   }
   CU(cudaMalloc((void **)&s->sc.partial, sizeof(double) * 2 * (size_t)maxt));
   s->sc.npartial = 2 * (long)maxt;
   CU(cudaMalloc((void **)&s->sc.counter, sizeof(unsigned int)));
   CU(cudaMemset(s->sc.counter, 0, sizeof(unsigned int)));
   CU(cudaMalloc((void **)&s->sc.box_norm, sizeof(double) * (size_t)maxbox));
   CU(cudaMalloc((void **)&s->d_norms, sizeof(double) * N_SLOTS * (size_t)(h->nlev + 1)));
   CU(cudaMemset(s->d_norms, 0, sizeof(double) * N_SLOTS * (size_t)(h->nlev + 1)));
   CU(cudaMalloc((void **)&s->d_citers, sizeof(int)));
   s->snap_points = snap_pts;
   CU(cudaMalloc((void **)&s->d_snap, sizeof(double) * 2 * (size_t)s->nvar * (size_t)(snap_pts ? snap_pts : 1)));
   CU(cudaMallocHost((void **)&s->h_res, sizeof(double) * 4));
   CU(cudaMalloc((void **)&s->d_hist, sizeof(double) * (size_t)(h->prm.max_iter > 0 ? h->prm.max_iter : 1)));
   CU(cudaMalloc((void **)&s->d_it, sizeof(int)));
   CU(cudaMalloc((void **)&s->d_parity, sizeof(int)));
   CU(cudaMemset(s->d_parity, 0, sizeof(int)));
   return 0;
}

const pgb_dop *pgb_operator_device_form(const pgb_operator *op);

void pgb_default_create_args(pgb_create_args *a)
{
   int k;
   memset(a, 0, sizeof(*a));
   pgb_default_params(&a->params);
   a->min_level = 1;
   a->nvar = 1;
   for (k = 0; k < PGB_NSRC_MAX; k++) a->restr_src[k] = PGB_HW_RESTR;
}

int pgb_create_ex(const pgb_create_args *a, pgb_solver **out)
{
   pgb_solver *s;
   pgb_hparams hp;
   const pgb_mg_params *params = &a->params;
   int rc, k, nsrc, v;
   const int nvar = a->nvar > 1 ? a->nvar : 1;
   const pgb_operator *ops[PGB_NVAR_MAX];
   *out = 0;
   if (!a->op) return fail(1, "no level operator (pgb_operator_create / pgb_operator_builtin)");
   if (nvar > PGB_NVAR_MAX) return fail(1, "at most %d elliptic variables", PGB_NVAR_MAX);
   ops[0] = a->op;
   nsrc = pgb_operator_device_form(a->op)->nsrc;
   for (v = 0; v < nvar; v++) {
      if (v) {
         if (!a->var_op[v]) return fail(1, "no operator for elliptic variable %d", v);
         ops[v] = a->var_op[v];
         if (pgb_operator_device_form(ops[v])->nsrc > nsrc) nsrc = pgb_operator_device_form(ops[v])->nsrc;
      }
      if (pgb_operator_vars(ops[v]) > nvar)
         return fail(1, "the operator of variable %d names u%d, beyond the %d variable(s)", v,
                     pgb_operator_vars(ops[v]) - 1, nvar);
   }
   if (params->interp_order != 2 && params->interp_order != 4)
      return fail(1, "interp_order must be 2 or 4");
   if (params->restr_u < 0 || params->restr_u > 3 || params->restr_res < 0 ||
       params->restr_res > 3 || params->restr_src < 0 || params->restr_src > 3)
      return fail(1, "restriction operators must be 0..3");
   for (k = 1; k < nsrc; k++)
      if (a->restr_src[k] < 0 || a->restr_src[k] > 3) return fail(1, "restriction operators must be 0..3");
   if (params->precision != PGB_FP64 && params->precision != PGB_MIXED)
      return fail(1, "precision must be PGB_FP64 or PGB_MIXED");
   s = (pgb_solver *)calloc(1, sizeof(*s));
   if (!s) return fail(10, "out of host memory");
   s->dop = *pgb_operator_device_form(a->op);
   s->nsrc = nsrc > 1 ? nsrc : 1;
   s->nvar = nvar;
   for (v = 0; v < nvar; v++) {   /* every variable's program reads the solver's sources */
      s->dops[v] = *pgb_operator_device_form(ops[v]);
      s->dops[v].nsrc = s->nsrc;
      if (nvar > 1) {   /* the program path handles the coupling */
         s->dops[v].kind = PGB_OPK_PROGRAM;
         s->dops[v].nvread = nvar;
         s->dops[v].cfixed = !getenv("PGB_COUPLINGS_EVERY_PASS") && pgb_dop_couplings_fixed(&s->dops[v]);
         s->dops[v].jfixed = !getenv("PGB_COUPLINGS_EVERY_PASS") && pgb_dop_jac_fixed(&s->dops[v]);
      }
   }
   if (nvar > 1) s->dop.kind = PGB_OPK_PROGRAM;
   memset(&hp, 0, sizeof(hp));
   hp.pre_swp = params->pre_swp;
   hp.pst_swp = params->pst_swp;
   hp.max_iter = params->max_iter;
   hp.min_iter = params->min_iter;
   hp.max_citer = params->max_citer;
   hp.tol = params->tol;
   hp.crtol = params->crtol;
   hp.w0_r = params->w0_r;
   hp.w0_i = params->w0_i;
   hp.min_cwidth = params->min_cwidth;
   hp.restr_u = params->restr_u;
   hp.restr_res = params->restr_res;
   hp.restr_src = params->restr_src;
   hp.interp_order = params->interp_order;
   hp.interp_buffer = params->interp_buffer;
   hp.precision = params->precision;
   hp.nsrc = s->nsrc;
   hp.restr_srck[0] = params->restr_src;
   for (k = 1; k < PGB_NSRC_MAX; k++) hp.restr_srck[k] = a->restr_src[k];
   hp.min_level = a->min_level > 0 ? a->min_level : 1;
   hp.nvar = nvar;
   rc = pgb_hier_build(&s->h, a->dim, s->dop.kind, a->base_shape, a->base_bbox, a->ngrids, a->grid_level,
                       a->grid_bbox, &hp);
   if (rc) {
      fail(2, "hierarchy: %s", s->h.err);
      pgb_hier_free(&s->h);
      free(s);
      return 2;
   }
   s->host_only = (a->flags & PGB_HOST_ONLY) != 0;
   if (!s->host_only && (rc = setup_device(s))) {
      pgb_destroy(s);
      return rc;
   }
   *out = s;
   return 0;
}

int pgb_create(int dim, int pde, const int *base_shape, const double *base_bbox, int ngrids,
               const int *grid_level, const double *grid_bbox, const pgb_mg_params *params,
               int flags, pgb_solver **out)
{
   pgb_create_args a;
   pgb_operator *op = 0;
   int rc, d;
   *out = 0;
   if (pde < 0 || pde > 2) return fail(1, "unknown pde kind %d", pde);
   if (pgb_operator_builtin(pde, &op)) return fail(1, "%s", g_err);
   pgb_default_create_args(&a);
   a.dim = dim;
   a.op = op;
   for (d = 0; d < 3; d++) a.base_shape[d] = d < dim ? base_shape[d] : 1;
   for (d = 0; d < 6; d++) a.base_bbox[d] = d < 2 * dim ? base_bbox[d] : 0;
   a.ngrids = ngrids;
   a.grid_level = grid_level;
   a.grid_bbox = grid_bbox;
   a.params = *params;
   a.flags = flags;
   rc = pgb_create_ex(&a, out);
   pgb_operator_destroy(op);
   return rc;
}

int pgb_destroy(pgb_solver *s)
{
   int L;
   if (!s) return 0;
   if (!s->host_only) {
      for (L = 1; L <= s->h.nlev; L++) {
         free_plan_dev(&s->h.sync[L][0]);
         free_plan_dev(&s->h.sync[L][1]);
         free_plan_dev(&s->h.sync_coarsest[L]);
         free_plan_dev(&s->h.inject[L]);
         free_plan_dev(&s->h.inject_init[L]);
         free_plan_dev(&s->h.interp[L]);
         if (s->d_tables[L]) cudaFree(s->d_tables[L]);
         if (s->d_snap_off[L]) cudaFree(s->d_snap_off[L]);
      }
      if (s->arena) cudaFree(s->arena);
      if (s->d_dop) cudaFree(s->d_dop);
      if (s->dbox) cudaFree(s->dbox);
      for (L = 1; L < PGB_NVAR_MAX; L++)
         if (s->vbox[L]) cudaFree(s->vbox[L]);
      if (s->d_vdop) cudaFree(s->d_vdop);
      if (s->sc.partial) cudaFree(s->sc.partial);
      if (s->sc.counter) cudaFree(s->sc.counter);
      if (s->sc.box_norm) cudaFree(s->sc.box_norm);
      if (s->d_norms) cudaFree(s->d_norms);
      if (s->d_citers) cudaFree(s->d_citers);
      if (s->d_snap) cudaFree(s->d_snap);
      if (s->d_trace) cudaFree(s->d_trace);
      if (s->h_res) cudaFreeHost(s->h_res);
      if (s->d_hist) cudaFree(s->d_hist);
      if (s->d_it) cudaFree(s->d_it);
      if (s->d_parity) cudaFree(s->d_parity);
      if (s->d_tmaps) cudaFree(s->d_tmaps);
      if (s->d_err) cudaFree(s->d_err);
      if (s->graph_ok) cudaGraphExecDestroy(s->gexec);
      if (s->solve_ok > 0) cudaGraphExecDestroy(s->sexec);
      if (s->prep_ok > 0) cudaGraphExecDestroy(s->pexec);
      if (s->stream) {
         cudaEventDestroy(s->ev0);
         cudaEventDestroy(s->ev1);
         cudaStreamDestroy(s->stream);
      }
      if (s->side) {
         cudaEventDestroy(s->evfork);
         cudaEventDestroy(s->evjoin);
         cudaStreamDestroy(s->side);
      }
   }
   free(s->hbox);
   free(s->tail);
   if (s->d_tailbar) cudaFree(s->d_tailbar);
   pgb_hier_free(&s->h);
   free(s);
   return 0;
}

void *pgb_stream(pgb_solver *s) { return (void *)s->stream; }

/* ---------------------------------------------------------------- data -- */
static int grid_box(const pgb_solver *s, int grid, const pgb_hbox **b)
{
   if (grid < 0 || grid >= s->h.ngrids) return fail(3, "grid %d out of range", grid);
   if (s->h.grid_box[grid] < 0)
      return fail(3, "grid %d lies below the hierarchy's coarsest AMR level %d", grid, s->h.prm.min_level);
   *b = &s->h.boxes[s->h.grid_box[grid]];
   return 0;
}

int pgb_grid_shape(const pgb_solver *s, int grid, int *shape3)
{
   const pgb_hbox *b = 0;
   if (grid_box(s, grid, &b)) return 3;
   memcpy(shape3, b->shape, sizeof(int) * 3);
   return 0;
}

static int copy_grid(pgb_solver *s, int grid, const double *u, const double *src, double *uout,
                     enum cudaMemcpyKind kin, enum cudaMemcpyKind kout)
{
   const pgb_hbox *b = 0;
   const pgb_dbox *db;
   size_t n;
   if (s->host_only) return fail(4, "solver was created with PGB_HOST_ONLY");
   if (grid_box(s, grid, &b)) return 3;
   db = &s->hbox[s->h.grid_box[grid]];
   n = sizeof(double) * (size_t)b->shape[0] * b->shape[1] * b->shape[2];
   if (u) CU(cudaMemcpyAsync(db->f[PGB_F_U], u, n, kin, s->stream));
   if (src) CU(cudaMemcpyAsync(db->f[PGB_F_SRC], src, n, kin, s->stream));
   if (uout) {
      CU(cudaMemcpyAsync(uout, db->f[PGB_F_U], n, kout, s->stream));
      CU(cudaStreamSynchronize(s->stream));
   }
   return 0;
}

static int copy_source(pgb_solver *s, int grid, int k, const double *src, enum cudaMemcpyKind kin)
{
   const pgb_hbox *b = 0;
   const pgb_dbox *db;
   if (s->host_only) return fail(4, "solver was created with PGB_HOST_ONLY");
   if (grid_box(s, grid, &b)) return 3;
   if (k < 0 || k >= s->nsrc) return fail(3, "source %d: the operator reads %d source(s)", k, s->dop.nsrc);
   db = &s->hbox[s->h.grid_box[grid]];
   CU(cudaMemcpyAsync(db->f[PGB_SRC_FIELD(k)], src, sizeof(double) * (size_t)b->shape[0] * b->shape[1] * b->shape[2],
                      kin, s->stream));
   return 0;
}

int pgb_set_source(pgb_solver *s, int grid, int k, const double *src)
{
   int rc;
   s->prepared = 0;
   rc = copy_source(s, grid, k, src, cudaMemcpyHostToDevice);
   if (!rc) CU(cudaStreamSynchronize(s->stream));
   return rc;
}

int pgb_set_source_device(pgb_solver *s, int grid, int k, const double *src)
{
   s->prepared = 0;
   return copy_source(s, grid, k, src, cudaMemcpyDeviceToDevice);
}

/* elliptic variable v of an input grid, in (u) or out (uout) */
static int copy_var(pgb_solver *s, int grid, int v, const double *u, double *uout)
{
   const pgb_hbox *b = 0;
   const pgb_dbox *db;
   size_t n;
   if (s->host_only) return fail(4, "solver was created with PGB_HOST_ONLY");
   if (grid_box(s, grid, &b)) return 3;
   if (v < 0 || v >= s->nvar) return fail(3, "variable %d: the solver has %d", v, s->nvar);
   db = &s->hbox[s->h.grid_box[grid]];
   n = sizeof(double) * (size_t)b->shape[0] * b->shape[1] * b->shape[2];
   if (u) {
      s->prepared = 0;
      CU(cudaMemcpyAsync(db->f[PGB_FV(v, PGB_F_U)], u, n, cudaMemcpyHostToDevice, s->stream));
   }
   if (uout) CU(cudaMemcpyAsync(uout, db->f[PGB_FV(v, PGB_F_U)], n, cudaMemcpyDeviceToHost, s->stream));
   CU(cudaStreamSynchronize(s->stream));
   return 0;
}

int pgb_set_var(pgb_solver *s, int grid, int v, const double *u) { return copy_var(s, grid, v, u, 0); }
int pgb_get_var(pgb_solver *s, int grid, int v, double *u) { return copy_var(s, grid, v, 0, u); }

int pgb_set_grid(pgb_solver *s, int grid, const double *u, const double *src)
{
   int rc;
   s->prepared = 0;
   rc = copy_grid(s, grid, u, src, 0, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost);
   if (!rc) CU(cudaStreamSynchronize(s->stream));
   return rc;
}
int pgb_get_grid(pgb_solver *s, int grid, double *u)
{
   return copy_grid(s, grid, 0, 0, u, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost);
}
int pgb_set_grid_device(pgb_solver *s, int grid, const double *u, const double *src)
{
   s->prepared = 0;
   return copy_grid(s, grid, u, src, 0, cudaMemcpyDeviceToDevice, cudaMemcpyDeviceToDevice);
}
int pgb_get_grid_device(pgb_solver *s, int grid, double *u)
{
   return copy_grid(s, grid, 0, 0, u, cudaMemcpyDeviceToDevice, cudaMemcpyDeviceToDevice);
}

/* ------------------------------------------------------------- V-cycle -- */
static double *norm_slot(pgb_solver *s, int L, int k) { return s->d_norms + N_SLOTS * L + k; }

/* The mixed form's residual pass over the finest level with its norm (and
 * D = -res for the next pre-smoothing block): one pass, or with several
 * elliptic variables one pass over each variable's view and the norm over
 * all of them */
static int finest_residual32(pgb_solver *s, pgb_trace *trace)
{
   const int Lf = s->h.nlev;
   int v;
   if (s->nvar == 1) {
      KC32(pgb_k_residual_fast(s->dbox, s->lv[Lf], s->h.pde, s->sc, norm_slot(s, Lf, N_RESID), trace, 0, s->stream));
      return 0;
   }
   for (v = 0; v < s->nvar; v++)
      KC32(pgb_k_residual_fast(s->vbox[v], s->lv[Lf], s->h.pde, s->sc, 0, 0, 0, s->stream));
   KC32(pgb_k_norm_vars(s->dbox, s->lv[Lf], s->sc, norm_slot(s, Lf, N_RESID), trace, s->stream));
   return 0;
}

static int lvl_coarsest(const pgb_solver *s, int L)   /* is_coarsest amrd/mg.c:553-567 */
{
   int b;
   for (b = 0; b < s->h.lev[L].nbox; b++)
      if (s->h.boxes[s->h.lev[L].box[b]].coarsest) return 1;
   return 0;
}

static int relax(pgb_solver *s, int L, int slot)
{
   KC(pgb_k_relax(s->dbox, s->lv[L], s->h.pde, s->sc, norm_slot(s, L, slot), s->d_trace, s->stream));
   return 0;
}

static int sync_field(pgb_solver *s, const pgb_plan *p, int field)
{
   if (p->nops) KC(pgb_k_copy(s->dbox, p, field, s->stream));
   return 0;
}

/* the same for field f (U..RHS) of every elliptic variable */
static int sync_vars(pgb_solver *s, const pgb_plan *p, int f)
{
   int v;
   for (v = 0; v < s->nvar; v++)
      if (sync_field(s, p, PGB_FV(v, f))) return 11;
   return 0;
}

/* Autotuner of the mixed form, run once per solver at its first
 * pgb_prepare: for every smoothed level it times the level's smoothing
 * block (max(pre, post) FP32 sweeps) plus its FP64 residual pass for each
 * tile depth (8, 4, 2, 1 planes per 32 x 8 tile; 3-D only) and each sweep
 * kernel: two global-memory colour passes per sweep, one shared-memory
 * sweep per launch or, on levels without a sync between sweeps, two, the
 * one-pass z-marching sweep and (3-D, boxes relaxed on their whole
 * interior) the TMA-staged one-pass sweep with columns 60 or 28 wide and
 * 4 to 64 planes deep, and keeps the fastest. No choice changes a
 * computed value (the sweeps are the same Gauss-Seidel sweeps; only the
 * norm's summation order follows the tiles). PGB_AUTOTUNE=0 keeps the
 * defaults; PGB_SWEEP_FUSE=0..7 forces one sweep kernel on every level
 * (PGB_SWEEP_MTZ=4/8/16/32/64 the TMA columns' depth with 4 to 7). */
/* the column width of the TMA sweep kernels f = 4..7 */
static int mtx_of(int f)
{
   return f == 4 ? 60 : f == 5 ? 28 : f == 6 ? 24 : 56;
}

/* Time one candidate as the V-cycle runs it: eight smoothing blocks of `nsw`
 * sweeps, each with its residual pass, captured into a graph and replayed
 * (one warm-up replay, one timed). Timing direct launches instead would
 * measure the host's launch rate on small levels, where a launch's kernel
 * time is a few microseconds. */
static int time_candidate(pgb_solver *s, int L, int nsw, int f, float *ms)
{
   const pgb_hier *h = &s->h;
   cudaGraph_t g = 0;
   cudaGraphExec_t ge = 0;
   int r, bad = 0;
   CU(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
   for (r = 0; r < 8 && !bad; r++) {
      int slot = PGB_W32_E;
      bad = pgb_k_sweep32(s->dbox, s->lv[L], nsw, f, &slot, s->stream) ||
            pgb_k_residual_fast(s->dbox, s->lv[L], h->pde, s->sc, norm_slot(s, L, N_RESID), 0, 0, s->stream);
   }
   cudaError_t e = cudaStreamEndCapture(s->stream, &g);
   if (bad) {
      if (g) cudaGraphDestroy(g);
      return fail(11, "%s", pgb_dev_error32());
   }
   if (e == cudaSuccess) e = cudaGraphInstantiate(&ge, g, 0);
   if (e == cudaSuccess) e = cudaGraphLaunch(ge, s->stream);
   if (e == cudaSuccess) e = cudaEventRecord(s->ev0, s->stream);
   if (e == cudaSuccess) e = cudaGraphLaunch(ge, s->stream);
   if (e == cudaSuccess) e = cudaEventRecord(s->ev1, s->stream);
   if (e == cudaSuccess) e = cudaEventSynchronize(s->ev1);
   if (e == cudaSuccess) e = cudaEventElapsedTime(ms, s->ev0, s->ev1);
   if (ge) cudaGraphExecDestroy(ge);
   if (g) cudaGraphDestroy(g);
   if (e != cudaSuccess) return fail(10, "autotuner graph: %s", cudaGetErrorString(e));
   return 0;
}

static int fp64_level1(const pgb_solver *s);
static void coarsest_args(pgb_solver *s, int L, pgb_coarsest_args *a);

/* The small-level kernel (pgb_dev.h, pgb_k_tail) takes the V-cycle's passes
 * over MG levels 1..Lc: the largest Lc below the finest level such that
 * every level up to it has at most PGB_TAIL_POINTS points (6000 unless set:
 * a 17^3 grid; the FP64 passes of larger levels run faster spread over the
 * whole GPU than on one cluster), no sync between its boxes, and no coarsest
 * boxes above level 1, where one coarsest box fits the on-chip FP32 coarsest
 * loop; at least two levels. Those levels relax by colour passes (their
 * sweeps are not autotuned). Off unless PGB_TAIL=1: measured on GB300 it is
 * slower than the V-cycle's own graph of one launch per pass (a graph node
 * costs about what a barrier and one trip to L2 per step cost here), with
 * the same bits. PGB_TAIL_GRID=1 meets at a counter across one CTA per SM
 * instead of a cluster barrier; PGB_TAIL_SOLO=n runs the passes of levels
 * of at most n points in CTA 0 alone. */
static int tail_plan(pgb_solver *s)
{
   pgb_hier *h = &s->h;
   const char *env = getenv("PGB_TAIL"), *pts = getenv("PGB_TAIL_POINTS"), *sol = getenv("PGB_TAIL_SOLO");
   const int mini = env && !strcmp(env, "mini");
   const long maxp = pts ? atol(pts) : mini ? 1500 : 6000, maxsolo = sol ? atol(sol) : 0;
   size_t staged = 0;
   const int nsw = h->prm.pre_swp + h->prm.pst_swp;
   int L, b, Lc = 0, steps = 1;
   pgb_coarsest_args a;
   s->tail_lc = s->tail_solo = 0;
   s->tail_mini = 0;
   if (!env || (strcmp(env, "1") && !mini) || h->prm.precision != PGB_MIXED || s->nvar > 1 || h->nlev < 3 || fp64_level1(s))
      return 0;
   coarsest_args(s, 1, &a);
   if (a.ncoarse != 1 || a.smem_points <= 0 ||
       a.smem_points * (long)(sizeof(double) + 3 * sizeof(float) + sizeof(int)) > 200 * 1024)
      return 0;
   for (L = 1; L < h->nlev && L <= PGB_TAIL_MAXLEV; L++) {
      long n = 0;
      for (b = 0; b < h->lev[L].nbox; b++) {
         const pgb_hbox *bx = &h->boxes[h->lev[L].box[b]];
         n += (long)bx->shape[0] * bx->shape[1] * bx->shape[2];
      }
      if (n > maxp || h->sync[L][0].nops || h->sync[L][1].nops || (L > 1 && lvl_coarsest(s, L))) break;
      if (mini) {   /* the level's arrays in one CTA's shared memory, laid out as the kernel stages them */
         size_t add = 0;
         int f;
         for (b = 0; b < h->lev[L].nbox; b++) {
            const pgb_dbox *db = &s->hbox[h->lev[L].box[b]];
            const size_t np = (size_t)db->n[0] * db->n[1] * db->n[2];
            for (f = 0; f < PGB_NF; f++)
               if (db->f[f]) add += (np * 8 + 15) / 16 * 16;
            for (f = 0; f < PGB_NW32; f++)
               if (db->w32[f]) add += ((size_t)db->wz * db->n[2] * 4 + 15) / 16 * 16;
            add += 2 * ((np + 15) / 16 * 16);
         }
         if (staged + add > 150 * 1024 || (size_t)h->nbox * sizeof(pgb_dbox) > 32 * 1024) break;
         staged += add;
      }
      if (n <= maxsolo && s->tail_solo == L - 1) s->tail_solo = L;
      /* a bound on the steps a level adds (passes of the down and up sweep) */
      steps += 10 + 2 * nsw + h->inject[L].nbatch + 2 * h->interp[L].nbatch;
      if (steps > PGB_TAIL_MAXSTEP) break;
      Lc = L;
   }
   if (Lc < 2) return 0;
   if (s->tail_solo > Lc) s->tail_solo = Lc;
   if (mini) {
      /* recompute the staged bytes of exactly levels 1..Lc */
      staged = 0;
      for (L = 1; L <= Lc; L++)
         for (b = 0; b < h->lev[L].nbox; b++) {
            const pgb_dbox *db = &s->hbox[h->lev[L].box[b]];
            const size_t np = (size_t)db->n[0] * db->n[1] * db->n[2];
            int f;
            for (f = 0; f < PGB_NF; f++)
               if (db->f[f]) staged += (np * 8 + 15) / 16 * 16;
            for (f = 0; f < PGB_NW32; f++)
               if (db->w32[f]) staged += ((size_t)db->wz * db->n[2] * 4 + 15) / 16 * 16;
            staged += 2 * ((np + 15) / 16 * 16);
         }
      s->tail_mini = staged;
      s->tail_ncta = 1;
   } else
      s->tail_ncta = pgb_tail_max_cluster((size_t)a.smem_points * (sizeof(double) + 3 * sizeof(float) + sizeof(int)));
   if (s->tail_ncta < 1) return 0;
   {
      const char *gm = getenv("PGB_TAIL_GRID");
      s->tail_grid = gm && !strcmp(gm, "1") ? pgb_tail_grid_ctas() : 0;
      if (s->tail_grid && !s->d_tailbar && cudaMalloc((void **)&s->d_tailbar, sizeof(unsigned int)) != cudaSuccess)
         return fail(10, "small-level kernel: barrier counter");
   }
   if (!s->tail && !(s->tail = (pgb_tail_prog *)malloc(sizeof(pgb_tail_prog))))
      return fail(10, "small-level kernel: host buffer");
   s->tail_lc = Lc;
   for (L = 1; L <= Lc; L++) {
      s->fuse[L] = 0;
      /* one CTA walks a step's blocks in turn: tiles of the full depth make
       * them few (a 9^3 level is 4 tiles of 32 x 8 x 8 points) */
      if (mini && h->dim == 3 && s->lv[L].tz != PGB_TZ && level_tables(s, L, PGB_TZ)) return 10;
   }
   if (mini) drop_graph(s);
   return 0;
}

int pgb_tail_levels(const pgb_solver *s, int *cluster_ctas)
{
   if (cluster_ctas) *cluster_ctas = s->tail_lc ? s->tail_ncta : 0;
   return s->tail_lc;
}

static int autotune(pgb_solver *s)
{
   pgb_hier *h = &s->h;
   const char *env = getenv("PGB_AUTOTUNE"), *force = getenv("PGB_SWEEP_FUSE");
   int L, changed = 0;
   int nsw = h->prm.pre_swp > h->prm.pst_swp ? h->prm.pre_swp : h->prm.pst_swp;
   s->tuned = 1;
   if (s->nvar > 1) return 0;   /* several variables: one smoother (the coupled colour passes) */
   if (force && force[0] >= '0' && force[0] <= '7' && !force[1]) {
      /* one sweep shape on every level instead of the measured choice */
      for (L = s->tail_lc > 1 ? s->tail_lc + 1 : 2; L <= h->nlev; L++) {
         int can_fuse = !h->sync[L][0].nops && !h->sync[L][1].nops && nsw >= 2;
         int f = force[0] - '0';
         if (f == 3 && h->dim != 3) f = 1;
         if (f >= 6 && !can_fuse) f -= 2;
         if (f >= 4 && !level_tma_ok(s, L)) f = 1;
         s->fuse[L] = f == 2 && !can_fuse ? 1 : f;
         if (f >= 4) {
            const char *mz = getenv("PGB_SWEEP_MTZ");
            s->mtx[L] = mtx_of(f);
            s->mtz[L] = mz && (!strcmp(mz, "4") || !strcmp(mz, "8") || !strcmp(mz, "16") || !strcmp(mz, "32") ||
                               !strcmp(mz, "64"))
                           ? atoi(mz)
                           : 32;
            if (level_tables(s, L, s->lv[L].tz)) return 10;
         }
      }
      drop_graph(s);
      return 0;
   }
   if ((env && !strcmp(env, "0")) || nsw < 1) return 0;
   for (L = s->tail_lc > 1 ? s->tail_lc + 1 : 2; L <= h->nlev; L++) {
      static const int tzs[4] = {8, 4, 2, 1};
      static const int mzs[5] = {4, 8, 16, 32, 64};
      int ntz = h->dim == 3 ? 4 : 1, a, f, best_tz = s->lv[L].tz, best_f = s->fuse[L], best_mtx = 60, best_mtz = 32;
      int can_fuse = !h->sync[L][0].nops && !h->sync[L][1].nops && nsw >= 2;
      const int tma = level_tma_ok(s, L);
      float best = 1e30f;
      for (a = 0; a < ntz; a++) {
         if (h->dim == 3 && tzs[a] != s->lv[L].tz) {
            if (level_tables(s, L, tzs[a])) return 10;
            changed = 1;
         }
         /* candidates: f < 4 once each; the TMA-staged sweep (f 4, 5: columns
          * 60 or 28 wide) and two of them per launch (f 6, 7: columns 24 or
          * 56 wide) with columns of 4 to 64 planes */
         for (int c = 0; c <= (h->dim == 3 ? 23 : can_fuse ? 2 : 1); c++) {
            f = c < 4 ? c : 4 + (c - 4) / 5;
            if ((f == 2 || f >= 6) && !can_fuse) continue;
            if (f >= 4) {
               if (!tma) continue;
               s->mtx[L] = mtx_of(f);
               s->mtz[L] = mzs[(c - 4) % 5];
               if (level_tables(s, L, tzs[a])) return 10;
               changed = 1;
            }
            float ms = 0;
            if (time_candidate(s, L, nsw, f, &ms)) return 10;
            if (ms < best) {
               best = ms;
               best_tz = s->lv[L].tz;
               best_f = f;
               best_mtx = f >= 4 ? s->mtx[L] : 60;
               best_mtz = f >= 4 ? s->mtz[L] : 32;
            }
         }
      }
      if (best_tz != s->lv[L].tz || s->mtx[L] != best_mtx || s->mtz[L] != best_mtz) {
         s->mtx[L] = best_mtx;
         s->mtz[L] = best_mtz;
         if (level_tables(s, L, best_tz)) return 10;
         changed = 1;
      }
      s->fuse[L] = best_f;
   }
   if (changed) drop_graph(s);
   return 0;
}

int pgb_level_tuning(pgb_solver *s, int L, int *tile_planes, int *sweeps_per_launch)
{
   if (s->host_only) return fail(4, "solver was created with PGB_HOST_ONLY");
   if (L < 1 || L > s->h.nlev) return fail(3, "level %d out of range", L);
   if (tile_planes) *tile_planes = s->lv[L].tz;
   if (sweeps_per_launch && L <= s->tail_lc)   /* relaxed inside the small-level kernel */
      *sweeps_per_launch = 8;
   else if (sweeps_per_launch)   /* the sweep mode (pamr_gb300.h lists them) */
      *sweeps_per_launch = (s->fuse[L] == 2 && (s->h.sync[L][0].nops || s->h.sync[L][1].nops)) ? 1 : s->fuse[L];
   return 0;
}

/* initialisation the reference performs while building the MG hierarchy
 * (build_mgh src/gh.c:1222-1365): MG-only grid functions start at zero and
 * pure MG levels receive u and the source by TF_MGH_INIT injection; with
 * PGB_PREPARE_KEEP_MG_DATA the MG-only levels keep the u and sources the
 * caller stored (pgb_box_set), as an existing MG hierarchy holds them
 * between vcycle calls (amrd/evolve.c:471-487) */
int pgb_prepare_ex(pgb_solver *s, int flags)
{
   int L;
   const int keep = (flags & PGB_PREPARE_KEEP_MG_DATA) != 0;
   if (s->host_only) return fail(4, "solver was created with PGB_HOST_ONLY");
   for (L = 1; L <= s->h.nlev; L++) {
      int mask = PGB_VMASK(s->nvar, PGB_F_RES) | PGB_VMASK(s->nvar, PGB_F_LOP) | PGB_VMASK(s->nvar, PGB_F_RHS);
      if (!s->h.lev[L].in_amrh && !keep) mask |= PGB_VMASK(s->nvar, PGB_F_U) | PGB_SRC_MASK(s->nsrc);
      KC(pgb_k_clear(s->dbox, s->lv[L], mask, s->stream));
   }
   for (L = s->h.nlev - 1; L >= 1 && !keep; L--)
      if (s->h.inject_init[L].nops) KC(pgb_k_restrict(s->dbox, &s->h.inject_init[L], ~0, 0, s->stream));
   /* With the caller's MG-level data, the sources of the pure MG levels are
    * still injected from the level above, top down: the reference's vcycle
    * does so in its down sweep (PAMR_inject into a level outside the AMR
    * hierarchy takes every variable's mg_inject, PAMR_TF_INJECT_TO_MG_LEV,
    * src/pamr.c:667-685, 1886-1893), which matters when the caller changed
    * the sources above since the hierarchy was built; the V-cycle itself
    * leaves this injection out because within one solve it rewrites the
    * same values. */
   for (L = s->h.nlev - 1; L >= 1 && keep; L--)
      if (!s->h.lev[L].in_amrh && s->h.inject_init[L].nops)
         KC(pgb_k_restrict(s->dbox, &s->h.inject_init[L], PGB_SRC_MASK(s->nsrc), 0, s->stream));
   if (s->h.prm.precision == PGB_MIXED) {
      if (!s->tuned) {
         int rc = tail_plan(s);
         if (!rc) rc = autotune(s);
         if (rc) return rc;
      }
      /* FP32 correction arrays start at 0 (D stays 0 wherever res is never
       * computed); the finest level's first pre-smoothing defect is the
       * initial residual */
      for (L = 1; L <= s->h.nlev; L++) {
         int v;
         KC(pgb_k_clear(s->dbox, s->lv[L],
                        PGB_VMASK(s->nvar, PGB_F_RES) | PGB_VMASK(s->nvar, PGB_F_LOP) | PGB_VMASK(s->nvar, PGB_F_RHS),
                        s->stream));
         for (v = 0; v < s->nvar; v++) {
            if (pgb_k_zero32(s->vbox[v], s->lv[L], s->stream)) return fail(11, "%s", pgb_dev_error32());
            if (s->nvar > 1 && (s->dops[v].cfixed || s->dops[v].jfixed) &&
                pgb_k_couplings(s->vbox[v], s->lv[L], s->stream))
               return fail(11, "%s", pgb_dev_error32());
         }
      }
      /* A level's residual is restricted from its FP32 copy D = -res when no
       * sync writes res there and the restriction of res is full weighting
       * (D is 0 wherever res is not computed). The V-cycle's clear of res
       * then only protects FP64 reads of res at points not rewritten in the
       * same cycle, and there are none: the FAS right-hand side reads res
       * at child-covered points, which the restriction rewrites first
       * (test_plans.py checks that inclusion); the coarse correction and
       * the interpolation rewrite what the interpolation and the update
       * read. Such levels skip the clear; pgb_prepare clears once. */
      for (L = 1; L <= s->h.nlev; L++) {
         const pgb_hier *h = &s->h;
         int i, ok = L == 1 || !h->sync[L][0].nops;
         if (L > 1)
            for (i = 0; i < h->inject[L - 1].nops && ok; i++) {
               const int op = ((const pgb_restrict_op *)h->inject[L - 1].h_ops)[i].op[PGB_F_RES];
               if (op != 0 && op != 3) ok = 0;
            }
         s->res32[L] = ok && s->nvar == 1;   /* several variables: res is restricted in FP64 */
      }
      if (finest_residual32(s, 0)) return 11;
      /* Levels below the finest whose cover tiles are a minority, with no
       * sync between boxes: between a post-smoothing and the next
       * pre-smoothing their points outside the cover tiles do not change,
       * so the pre-smoothing defect there is carried over in FP32; the
       * first one is computed here. */
      for (L = 2; L < s->h.nlev; L++) {
         const pgb_hier *h = &s->h;
         /* not on levels with coarsest boxes: their coarsest-grid loop
          * changes u after the post-smoothing, so D cannot be carried */
         s->dnext[L] = s->nvar == 1 && h->prm.pre_swp > 0 && !h->sync[L][0].nops && !h->sync[L][1].nops &&
                       2 * s->lv[L].nctiles < s->lv[L].ntiles && !lvl_coarsest(s, L);
         if (s->dnext[L] &&
             pgb_k_fas_defect(s->dbox, s->lv[L], h->pde, h->prm.w0_r, 0, s->stream))
            return fail(11, "%s", pgb_dev_error32());
      }
   }
   CU(cudaMemsetAsync(s->d_citers, 0, sizeof(int), s->stream));
   CU(cudaMemsetAsync(s->d_parity, 0, sizeof(int), s->stream));   /* every solve starts on an even cycle */
   s->prepared = 1;
   return 0;
}

int pgb_prepare(pgb_solver *s) { return pgb_prepare_ex(s, 0); }

/* ------------------------------------------------------ box-level data -- */
/* field of pgb_box_set / pgb_box_get -> grid function */
static int box_field(const pgb_solver *s, int field, int *f)
{
   if (field == PGB_FIELD_U) *f = PGB_F_U;
   else if (field == PGB_FIELD_RES) *f = PGB_F_RES;
   else if (field == PGB_FIELD_LOP) *f = PGB_F_LOP;
   else if (field == PGB_FIELD_RHS) *f = PGB_F_RHS;
   else if (field >= PGB_FIELD_SRC && field < PGB_FIELD_SRC + s->nsrc) *f = PGB_SRC_FIELD(field - PGB_FIELD_SRC);
   else if (field >= PGB_FIELD_VAR(1) && field < PGB_FIELD_VAR(s->nvar))   /* variables 1.. */
      *f = PGB_FV(1 + (field - PGB_FIELD_VAR(1)) / 4, PGB_F_U + (field - PGB_FIELD_VAR(1)) % 4);
   else return fail(3, "unknown field %d", field);
   return 0;
}

static int box_copy(pgb_solver *s, int L, int idx, int field, const double *in, double *out)
{
   const pgb_hbox *b;
   int f = 0;
   size_t n;
   if (s->host_only) return fail(4, "solver was created with PGB_HOST_ONLY");
   if (L < 1 || L > s->h.nlev || idx < 0 || idx >= s->h.lev[L].nbox) return fail(3, "no box %d on level %d", idx, L);
   if (box_field(s, field, &f)) return 3;
   b = &s->h.boxes[s->h.lev[L].box[idx]];
   n = sizeof(double) * (size_t)b->shape[0] * b->shape[1] * b->shape[2];
   if (in) {
      s->prepared = 0;
      CU(cudaMemcpyAsync(s->hbox[s->h.lev[L].box[idx]].f[f], in, n, cudaMemcpyHostToDevice, s->stream));
   } else
      CU(cudaMemcpyAsync(out, s->hbox[s->h.lev[L].box[idx]].f[f], n, cudaMemcpyDeviceToHost, s->stream));
   CU(cudaStreamSynchronize(s->stream));
   return 0;
}

int pgb_box_set(pgb_solver *s, int L, int idx, int field, const double *in)
{
   return box_copy(s, L, idx, field, in, 0);
}

int pgb_box_get(pgb_solver *s, int L, int idx, int field, double *out)
{
   return box_copy(s, L, idx, field, 0, out);
}


/* one smoothing block of the FP64 form (nsweep Newton-GS sweeps + syncs,
 * amrd/mg.c:135-141 / 161-167) */
static int smooth(pgb_solver *s, int L, int nsweep, int slot)
{
   pgb_hier *h = &s->h;
   int it;
   for (it = 0; it < nsweep; it++) {
      if (relax(s, L, slot)) return 11;
      if (sync_vars(s, &h->sync[L][it ? 1 : 0], PGB_F_U)) return 11;
   }
   return 0;
}

/* fills the coarsest-grid loop's arguments for level L */
/* the mixed form smooths MG level 1 in FP64 exactly as the FP64 form does
 * (pre- and post-smoothing, then the reference's coarsest-grid loop) when
 * it holds several coarsest grids: the islands a refined level's grids
 * coarsen to, often thin strips, for which the FP32 SOR defect correction
 * of one grid is no substitute */
static int fp64_level1(const pgb_solver *s)
{
   int b, n = 0;
   for (b = 0; b < s->h.lev[1].nbox; b++) n += s->h.boxes[s->h.lev[1].box[b]].coarsest != 0;
   return s->h.prm.precision == PGB_MIXED && n > 1;
}

static void coarsest_args(pgb_solver *s, int L, pgb_coarsest_args *a)
{
   pgb_hier *h = &s->h;
   const pgb_hparams *p = &h->prm;
   int b, mixed = p->precision == PGB_MIXED && !(L == 1 && fp64_level1(s)), nmax = 0, d;
   memset(a, 0, sizeof(*a));
   a->start_iter = mixed ? 0 : p->pst_swp;
   a->max_citer = p->max_citer;
   a->crtol = p->crtol;
   a->res_dn = norm_slot(s, L, p->pre_swp > 0 ? N_RELAX_DN : N_COARSE);
   a->res_out = norm_slot(s, L, N_COARSE);
   a->iters_out = s->d_citers;
   for (b = 0; b < h->lev[L].nbox; b++) {
      const pgb_hbox *bx = &h->boxes[h->lev[L].box[b]];
      if (!bx->coarsest) continue;
      a->smem_points += (long)bx->shape[0] * bx->shape[1] * bx->shape[2];
      a->ncoarse++;
      for (d = 0; d < h->dim; d++)
         if (bx->shape[d] > nmax) nmax = bx->shape[d];
   }
   a->stagnation_exit = mixed;
   a->ctol_from_first = mixed;
   a->sor = mixed && s->nvar > 1;
   /* red-black SOR factor of the model problem, 2/(1 + sin(pi h)) */
   a->omega = nmax > 3 ? 2.0 / (1.0 + sin(3.141592653589793 / (nmax - 1))) : 1.0;
   {
      /* enough sweeps for the SOR error (about k (omega-1)^k after k sweeps)
       * to fall below crtol/4 in one correction */
      double rho = a->omega - 1.0 > 0.2 ? a->omega - 1.0 : 0.2, tgt = p->crtol > 0 ? p->crtol / 4 : 1e-6;
      int m = (int)ceil(log(tgt) / log(rho)) + 3;
      a->inner_sweeps = m < 2 ? 2 : m > 64 ? 64 : m;
   }
   a->snap = s->d_snap;
   a->snap_points = s->snap_points;
   a->snap_off = s->d_snap_off[L];
}

static int vcycle_fp64(pgb_solver *s)
{
   pgb_hier *h = &s->h;
   const pgb_hparams *p = &h->prm;
   int L, Lf = h->nlev;
   /* clear_MG_vars(Lf) amrd/mg.c:91 */
   const int nv = s->nvar;
   KC(pgb_k_clear(s->dbox, s->lv[Lf],
                  PGB_VMASK(nv, PGB_F_RES) | PGB_VMASK(nv, PGB_F_RHS) | PGB_VMASK(nv, PGB_F_LOP), s->stream));
   for (L = Lf; L > 0; L--) {
      if (L < Lf) {
         KC(pgb_k_residual(s->dbox, s->lv[L + 1], h->pde, s->sc, norm_slot(s, L + 1, N_RESID),
                           s->d_trace, s->stream));
         if (sync_vars(s, &h->sync[L + 1][0], PGB_F_RES)) return 11;   /* set_res_sync */
         /* clear_MG_vars(L): rhs and lop are rewritten by lop_rhs below */
         KC(pgb_k_clear(s->dbox, s->lv[L], PGB_VMASK(nv, PGB_F_RES), s->stream));
         /* the source restriction of MG-only levels (TF_INJECT_TO_MG_LEV) is left
          * out: it reads and writes the same values every cycle, and
          * pgb_prepare's build-time injection (same ops, same operator) has
          * already put them in place */
         if (h->inject[L].nops) KC(pgb_k_restrict(s->dbox, &h->inject[L], ~PGB_SRC_MASK(s->nsrc), 0, s->stream));
         if (sync_vars(s, &h->sync[L][0], PGB_F_U)) return 11;
         KC(pgb_k_lop_rhs(s->dbox, s->lv[L], h->pde, p->w0_r, s->stream));
      }
      if (smooth(s, L, p->pre_swp, N_RELAX_DN)) return 11;
   }
   for (L = 1; L <= Lf; L++) {
      if (L > 1) {
         KC(pgb_k_cgc_coarse(s->dbox, s->lv[L - 1], p->w0_i, s->stream));
         for (int v = 0; v < nv && h->interp[L].nops; v++)
            KC(pgb_k_interp(s->dbox, &h->interp[L], PGB_FV(v, PGB_F_RES), h->dim, s->stream));
         KC(pgb_k_add_res(s->dbox, s->lv[L], s->stream));
      }
      if (smooth(s, L, p->pst_swp, N_RELAX_UP)) return 11;
      if (lvl_coarsest(s, L)) {
         pgb_coarsest_args a;
         coarsest_args(s, L, &a);
         KC(pgb_k_coarsest(s->dbox, s->lv[L], h->pde, &h->sync_coarsest[L], a, s->d_trace, s->stream));
      }
      if (L == Lf)
         KC(pgb_k_residual(s->dbox, s->lv[Lf], h->pde, s->sc, norm_slot(s, Lf, N_RESID), s->d_trace,
                           s->stream));
   }
   return 0;
}

/* FP32 sweeps on the correction E of level L, synced between boxes like u,
 * over the box table `boxes` (the solver's, or a variable's view); the
 * block starts from slot *slot, which receives the slot it ends in */
static int sweeps32_on(pgb_solver *s, const pgb_dbox *boxes, int L, int nsweep, int *slot)
{
   pgb_hier *h = &s->h;
   int it;
   if (!h->sync[L][0].nops && !h->sync[L][1].nops) {
      KC32(pgb_k_sweep32(boxes, s->lv[L], nsweep, s->fuse[L], slot, s->stream));
      return 0;
   }
   for (it = 0; it < nsweep; it++) {
      KC32(pgb_k_sweep32(boxes, s->lv[L], 1, s->fuse[L] == 2 ? 1 : s->fuse[L], slot, s->stream));
      if (h->sync[L][it ? 1 : 0].nops)
         KC32(pgb_k_copy32(boxes, &h->sync[L][it ? 1 : 0], *slot, s->stream));
   }
   return 0;
}

static int sweeps32(pgb_solver *s, int L, int nsweep, int *slot) { return sweeps32_on(s, s->dbox, L, nsweep, slot); }

/* the FP32 defect carry and the update of a block in one kernel (where the
 * update's zeros go to the slot the defect does not read); PGB_NO_FUSED_UPDATE=1
 * keeps the two kernels */
static int fused_update(const pgb_solver *s)
{
   (void)s;
   return !getenv("PGB_NO_FUSED_UPDATE");
}

/* Levels whose residual is restricted from its FP32 copy (no sync of res)
 * carry the defect after pre-smoothing in FP32, D - (lap E + C E) before the
 * update (k_defect32), instead of a fresh FP64 residual: nothing reads that
 * level's FP64 res at relaxed points. The carried defect is exact up to
 * FP32 rounding relative to the defect of this cycle, because D is
 * recomputed in FP64 on the whole level once per cycle: by the FAS pass
 * below the finest level, by the residual that ends the cycle on the
 * finest. Levels that carry D across cycles outside their cover tiles
 * (dnext) keep the FP64 residual: two carries in a row would let FP32
 * rounding of early, large defects accumulate there. */
static int defect32_level(const pgb_solver *s, int L)
{
   return L > 1 && s->res32[L] && !s->dnext[L] && s->h.prm.pre_swp > 0;
}

/* The dnext levels among them alternate: on even cycles of a solve the
 * FP64 residual after pre-smoothing refreshes D on the whole level, on odd
 * cycles D is carried in FP32 as above. Between two refreshes D is then
 * carried through four updates, whose FP32 rounding stays far below the
 * defect of the cycle. A device flag (d_parity, flipped at the end of each
 * cycle) gates the two passes, so one captured cycle serves both. */
static int alt_level(const pgb_solver *s, int L)
{
   return L > 1 && s->res32[L] && s->dnext[L] && s->h.prm.pre_swp > 0;
}

/* The mixed form of the V-cycle (same transfers and the same FP64 residual,
 * restriction and norm as vcycle_fp64; the arithmetic of each smoothing
 * block is described in pgb_kernels32.cu). The finest level's pre-smoothing
 * defect is the residual the previous cycle ended with (pgb_prepare
 * computes the first); the coarsest level is smoothed by the coarsest-grid
 * loop alone. */
static int vcycle_mixed(pgb_solver *s)
{
   pgb_hier *h = &s->h;
   const pgb_hparams *p = &h->prm;
   int L, Lf = h->nlev;
   /* levels 1..tail_lc as steps of one small-level kernel (recorded from
    * the FAS pass of level tail_lc on the way down to its update on the way
    * up; not while norms are traced) */
   const int tail = s->tail_lc > 1 && !s->d_trace ? s->tail_lc : 0;
   /* clear_MG_vars: only where an FP64 read could see a value of an earlier
    * cycle (see pgb_prepare) */
   if (!s->res32[Lf])
      KC(pgb_k_clear(s->dbox, s->lv[Lf], (1 << PGB_F_RES) | (1 << PGB_F_RHS) | (1 << PGB_F_LOP), s->stream));
   for (L = Lf; L > 0; L--) {
      if (L < Lf) {
         pgb_tail_set_solo(L + 1 <= s->tail_solo);   /* passes reading level L+1 */
         /* this norm is only ever traced (the finest level's convergence
          * norm comes from the residual after post-smoothing) */
         if (!defect32_level(s, L + 1))
            KC32(pgb_k_residual_fast(s->dbox, s->lv[L + 1], h->pde, s->sc,
                                     s->d_trace ? norm_slot(s, L + 1, N_RESID) : 0, s->d_trace,
                                     alt_level(s, L + 1) ? s->d_parity : 0, s->stream));
         if (sync_field(s, &h->sync[L + 1][0], PGB_F_RES)) return 11;
         if (!s->res32[L]) KC(pgb_k_clear(s->dbox, s->lv[L], 1 << PGB_F_RES, s->stream));
         if (h->inject[L].nops)
            KC(pgb_k_restrict(s->dbox, &h->inject[L], ~PGB_SRC_MASK(s->nsrc), s->res32[L + 1], s->stream));
         if (sync_field(s, &h->sync[L][0], PGB_F_U)) return 11;
         if (L == tail) pgb_tail_begin(s->tail, h->pde, h->nbox, s->tail_mini);
         pgb_tail_set_solo(L <= s->tail_solo);   /* passes over level L */
         if (L == 1) KC32(pgb_k_lop_rhs_fast(s->dbox, s->lv[L], h->pde, p->w0_r, s->stream));
         else KC32(pgb_k_fas_defect(s->dbox, s->lv[L], h->pde, p->w0_r, s->dnext[L], s->stream));
      }
      /* the correction slots: every cycle starts each level from E = 0 in
       * PGB_W32_E; the pre-smoothing block leaves E = 0 in the slot the
       * post-smoothing block starts from (the slot it ended in, or the other
       * one where its update also carries the defect), and that block
       * zeroes PGB_W32_E again (which the captured graph relies on) */
      s->eslot[L] = PGB_W32_E;
      if (L == 1 && fp64_level1(s) && smooth(s, 1, p->pre_swp, N_RELAX_DN)) return 11;
      if (L > 1 && p->pre_swp > 0) {
         int slot = PGB_W32_E;
         const int dmode = defect32_level(s, L) ? 1 : alt_level(s, L) ? 2 : 0;
         if (sweeps32(s, L, p->pre_swp, &slot)) return 11;
         if (dmode && s->fuse[L] > 0 && fused_update(s)) {   /* sweeps that alternate the slots */
            /* defect and update in one pass: E = 0 goes to the other slot,
             * where the post-smoothing block then starts */
            const int z = slot == PGB_W32_E ? PGB_W32_E2 : PGB_W32_E;
            KC32(pgb_k_update_defect(s->dbox, s->lv[L], 0, slot, z, 1, dmode == 2 ? s->d_parity : 0, 1,
                                     s->stream));
            s->eslot[L] = z;
         } else {
            if (dmode == 1) KC32(pgb_k_defect32(s->dbox, s->lv[L], slot, 0, 0, s->stream));
            else if (dmode == 2) KC32(pgb_k_defect32(s->dbox, s->lv[L], slot, s->d_parity, 1, s->stream));
            KC32(pgb_k_update(s->dbox, s->lv[L], 0, slot, slot, s->stream));
            s->eslot[L] = slot;
         }
         if (sync_field(s, &h->sync[L][1], PGB_F_U)) return 11;
      }
   }
   for (L = 1; L <= Lf; L++) {
      if (L > 1) {
         int slot = s->eslot[L];
         pgb_tail_set_solo(L <= s->tail_solo);   /* passes over levels L-1 and L */
         KC32(pgb_k_cgc_mixed(s->dbox, s->lv[L - 1], 1.0 / p->w0_i, s->stream));
         if (h->interp[L].nops)
            KC32(pgb_k_interp_mixed(s->dbox, &h->interp[L], h->dim, slot, s->stream, s->side, s->evfork,
                                    s->evjoin));
         if (sweeps32(s, L, p->pst_swp, &slot)) return 11;
         if (s->dnext[L] && slot != PGB_W32_E && fused_update(s)) {
            KC32(pgb_k_update_defect(s->dbox, s->lv[L], 1, slot, PGB_W32_E, 1, 0, 0, s->stream));
         } else {
            if (s->dnext[L]) KC32(pgb_k_defect32(s->dbox, s->lv[L], slot, 0, 0, s->stream));
            KC32(pgb_k_update(s->dbox, s->lv[L], 1, slot, PGB_W32_E, s->stream));
         }
         if (sync_field(s, &h->sync[L][1], PGB_F_U)) return 11;
      }
      if (L == 1 && fp64_level1(s) && smooth(s, 1, p->pst_swp, N_RELAX_UP)) return 11;
      /* the coarsest-grid loop (amrd/mg.c:172-190) wherever coarsest boxes
       * are: on MG level 1, and above it in hierarchies whose base has
       * several islands that stop coarsening at different levels (a
       * hierarchy built from a refined AMR level) */
      if (lvl_coarsest(s, L)) {
         pgb_coarsest_args a;
         int rc;
         coarsest_args(s, L, &a);
         /* the FP32 SOR defect correction is made for one coarsest grid;
          * several (islands of a refined level's grids, often thin strips)
          * take the FP64 Gauss-Seidel loop of the reference */
         rc = a.ncoarse == 1 && !(L == 1 && fp64_level1(s))
                 ? pgb_k_coarsest_mixed(s->dbox, s->lv[L], h->pde, &h->sync_coarsest[L], a, s->d_trace, s->stream)
                 : 1;
         if (rc < 0) return fail(11, "%s", pgb_dev_error32());
         if (rc > 0)   /* too large for one CTA's shared memory: the FP64 loop */
            KC(pgb_k_coarsest(s->dbox, s->lv[L], h->pde, &h->sync_coarsest[L], a, s->d_trace, s->stream));
      }
      if (L == tail) {
         if (pgb_tail_end()) return fail(11, "%s", pgb_dev_error32());
         s->tail->grid = s->tail_grid;
         s->tail->bar_cnt = s->d_tailbar;
         s->tail->err = s->d_err;
         KC32(pgb_k_tail(s->dbox, s->tail, s->tail_grid ? s->tail_grid : s->tail_ncta, s->sc, s->stream));
      }
      if (L == Lf)
         KC32(pgb_k_residual_fast(s->dbox, s->lv[Lf], h->pde, s->sc, norm_slot(s, Lf, N_RESID),
                                  s->d_trace, 0, s->stream));
   }
   for (L = 2; L <= Lf; L++)
      if (alt_level(s, L)) {
         KC32(pgb_k_flip(s->d_parity, s->stream));
         break;
      }
   return 0;
}

/* FP32 sweeps of the coupled smoother of several variables on level L
 * (colour passes in place on each variable's E, synced between boxes like
 * u) */
static int sweeps32_vars(pgb_solver *s, int L, int nsweep)
{
   pgb_hier *h = &s->h;
   pgb_vtabs vt;
   int it, v;
   memset(&vt, 0, sizeof(vt));
   for (v = 0; v < s->nvar; v++) vt.t[v] = s->vbox[v];
   for (it = 0; it < nsweep; it++) {
      KC32(pgb_k_relax32_vars(vt, s->lv[L], 0, s->stream));
      KC32(pgb_k_relax32_vars(vt, s->lv[L], 1, s->stream));
      for (v = 0; v < s->nvar && h->sync[L][it ? 1 : 0].nops; v++)
         KC32(pgb_k_copy32(s->vbox[v], &h->sync[L][it ? 1 : 0], PGB_W32_E, s->stream));
   }
   return 0;
}

/* The mixed V-cycle of several elliptic variables. The one-variable passes
 * run once per variable, over that variable's view of the boxes
 * (var_views): residual, FAS right-hand side (each also leaving the
 * variable's defect D, Jacobian term C and coupling coefficients), update,
 * coarse-grid correction and interpolation. The smoothing blocks are the
 * coupled FP32 smoother over all variables at once (k_relax32_vars: at each
 * point variable after variable, as the FP64 form's relax), which keeps the
 * smoothing of modes the coupling dominates, on coarse levels where s dx^2
 * is large; clears, restrictions and syncs run once over the box table with
 * every variable's fields, the coarsest grid takes the FP64 loop over all
 * variables and the norm sums every variable's residual. The FP32 defect
 * carry and FP32 residual restriction of the one-variable form, its fused
 * and TMA sweeps and the small-level kernel are left out. */
static int vcycle_mixed_vars(pgb_solver *s)
{
   pgb_hier *h = &s->h;
   const pgb_hparams *p = &h->prm;
   const int nv = s->nvar, Lf = h->nlev;
   int L, v;
   KC(pgb_k_clear(s->dbox, s->lv[Lf], PGB_VMASK(nv, PGB_F_RES) | PGB_VMASK(nv, PGB_F_RHS) | PGB_VMASK(nv, PGB_F_LOP),
                  s->stream));
   for (L = Lf; L > 0; L--) {
      if (L < Lf) {
         for (v = 0; v < nv; v++)
            KC32(pgb_k_residual_fast(s->vbox[v], s->lv[L + 1], h->pde, s->sc, 0, 0, 0, s->stream));
         if (s->d_trace)
            KC32(pgb_k_norm_vars(s->dbox, s->lv[L + 1], s->sc, norm_slot(s, L + 1, N_RESID), s->d_trace, s->stream));
         if (sync_vars(s, &h->sync[L + 1][0], PGB_F_RES)) return 11;
         KC(pgb_k_clear(s->dbox, s->lv[L], PGB_VMASK(nv, PGB_F_RES), s->stream));
         if (h->inject[L].nops) KC(pgb_k_restrict(s->dbox, &h->inject[L], ~PGB_SRC_MASK(s->nsrc), 0, s->stream));
         if (sync_vars(s, &h->sync[L][0], PGB_F_U)) return 11;
         for (v = 0; v < nv; v++) {
            if (L == 1) KC32(pgb_k_lop_rhs_fast(s->vbox[v], s->lv[L], h->pde, p->w0_r, s->stream));
            else KC32(pgb_k_fas_defect(s->vbox[v], s->lv[L], h->pde, p->w0_r, 0, s->stream));
         }
      }
      if (L == 1 && fp64_level1(s) && smooth(s, 1, p->pre_swp, N_RELAX_DN)) return 11;
      if (L > 1 && p->pre_swp > 0) {
         if (sweeps32_vars(s, L, p->pre_swp)) return 11;
         for (v = 0; v < nv; v++) KC32(pgb_k_update(s->vbox[v], s->lv[L], 0, PGB_W32_E, PGB_W32_E, s->stream));
         if (sync_vars(s, &h->sync[L][1], PGB_F_U)) return 11;
      }
   }
   for (L = 1; L <= Lf; L++) {
      if (L > 1) {
         for (v = 0; v < nv; v++) {
            KC32(pgb_k_cgc_mixed(s->vbox[v], s->lv[L - 1], 1.0 / p->w0_i, s->stream));
            if (h->interp[L].nops)
               KC32(pgb_k_interp_mixed(s->vbox[v], &h->interp[L], h->dim, PGB_W32_E, s->stream, s->side, s->evfork,
                                       s->evjoin));
         }
         if (sweeps32_vars(s, L, p->pst_swp)) return 11;
         for (v = 0; v < nv; v++) KC32(pgb_k_update(s->vbox[v], s->lv[L], 1, PGB_W32_E, PGB_W32_E, s->stream));
         if (sync_vars(s, &h->sync[L][1], PGB_F_U)) return 11;
      }
      if (L == 1 && fp64_level1(s) && smooth(s, 1, p->pst_swp, N_RELAX_UP)) return 11;
      if (lvl_coarsest(s, L)) {
         pgb_coarsest_args a;
         coarsest_args(s, L, &a);
         KC(pgb_k_coarsest(s->dbox, s->lv[L], h->pde, &h->sync_coarsest[L], a, s->d_trace, s->stream));
      }
      if (L == Lf && finest_residual32(s, s->d_trace)) return 11;
   }
   return 0;
}

static int vcycle_launch(pgb_solver *s)
{
   if (s->h.prm.precision != PGB_MIXED) return vcycle_fp64(s);
   if (s->nvar > 1) return vcycle_mixed_vars(s);
   const int rc = vcycle_mixed(s);
   if (rc && pgb_tail_recording()) pgb_tail_end();   /* an error inside the recorded levels */
   return rc;
}

/* The V-cycle's launches never depend on host-side values, so the whole
 * cycle (and the read-back of the finest residual) is captured once into a
 * CUDA graph and replayed: one launch per cycle instead of ~100. */
static int build_graph(pgb_solver *s)
{
   cudaGraph_t g = 0;
   cudaError_t e;
   long long before = pgb_dev_launches() + pgb_dev_launches32();
   int rc;
   CU(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
   rc = vcycle_launch(s);
   if (!rc && cudaMemcpyAsync(s->h_res, norm_slot(s, s->h.nlev, N_RESID), sizeof(double),
                              cudaMemcpyDeviceToHost, s->stream) != cudaSuccess)
      rc = fail(10, "graph capture: residual read-back");
   e = cudaStreamEndCapture(s->stream, &g);
   if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
   }
   if (e != cudaSuccess) return fail(10, "cudaStreamEndCapture: %s", cudaGetErrorString(e));
   e = cudaGraphInstantiate(&s->gexec, g, 0);
   cudaGraphDestroy(g);
   if (e != cudaSuccess) return fail(10, "cudaGraphInstantiate: %s", cudaGetErrorString(e));
   s->graph_kernels = pgb_dev_launches() + pgb_dev_launches32() - before;
   g_captured += s->graph_kernels;
   s->graph_ok = 1;
   return 0;
}

/* The whole solve loop as one graph: a conditional while node whose body
 * is one V-cycle and k_solve_step, which records the finest residual and
 * sets the condition exactly as pgb_solve's host loop would decide, so the
 * host waits once per solve instead of once per cycle. Where the runtime
 * refuses the node, solve_ok = -1 and pgb_solve keeps the host loop. */
static int build_solve_graph(pgb_solver *s)
{
   const pgb_hparams *p = &s->h.prm;
   cudaGraph_t g = 0, body;
   cudaGraphConditionalHandle hnd;
   cudaGraphNode_t node;
   struct cudaGraphNodeParams cp;
   cudaError_t e;
   int rc;
   long long before = pgb_dev_launches() + pgb_dev_launches32();
   if (cudaGraphCreate(&g, 0) != cudaSuccess) return fail(10, "cudaGraphCreate");
   memset(&cp, 0, sizeof(cp));
   if (cudaGraphConditionalHandleCreate(&hnd, g, 1, cudaGraphCondAssignDefault) != cudaSuccess) goto refused;
   cp.type = cudaGraphNodeTypeConditional;
   cp.conditional.handle = hnd;
   cp.conditional.type = cudaGraphCondTypeWhile;
   cp.conditional.size = 1;
   if (cudaGraphAddNode(&node, g, NULL, NULL, 0, &cp) != cudaSuccess) goto refused;
   body = cp.conditional.phGraph_out[0];
   if (cudaStreamBeginCaptureToGraph(s->stream, body, NULL, NULL, 0, cudaStreamCaptureModeThreadLocal) !=
       cudaSuccess)
      goto refused;
   rc = vcycle_launch(s);
   if (!rc && pgb_k_solve_step(hnd, norm_slot(s, s->h.nlev, N_RESID), s->d_hist, s->d_it, p->min_iter,
                               p->max_iter, p->tol, s->stream))
      rc = fail(10, "%s", pgb_dev_error32());
   e = cudaStreamEndCapture(s->stream, &body);
   g_captured += pgb_dev_launches() + pgb_dev_launches32() - before;   /* counted when replayed */
   if (rc) {
      cudaGraphDestroy(g);
      return rc;
   }
   if (e != cudaSuccess) goto refused;
   e = cudaGraphInstantiate(&s->sexec, g, 0);
   cudaGraphDestroy(g);
   if (e != cudaSuccess) {
      cudaGetLastError();
      s->solve_ok = -1;
      return 0;
   }
   s->solve_ok = 1;
   return 0;
refused:
   cudaGetLastError();
   cudaGraphDestroy(g);
   s->solve_ok = -1;
   return 0;
}

static void drop_graph(pgb_solver *s)
{
   if (s->graph_ok) cudaGraphExecDestroy(s->gexec);
   s->graph_ok = 0;
   if (s->solve_ok > 0) cudaGraphExecDestroy(s->sexec);
   s->solve_ok = 0;
   if (s->prep_ok > 0) cudaGraphExecDestroy(s->pexec);
   s->prep_ok = 0;
}

/* pgb_prepare's launches as one graph: every solve starts with the same
 * clears, injections and first residual (after the autotuner's one-time
 * timing, which is why the first pgb_prepare runs directly), so pgb_solve
 * replays them instead of issuing some thirty launches from the host. */
static int build_prepare_graph(pgb_solver *s)
{
   cudaGraph_t g = 0;
   cudaError_t e;
   int rc;
   if (cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      cudaGetLastError();
      s->prep_ok = -1;
      return 0;
   }
   rc = pgb_prepare(s);
   e = cudaStreamEndCapture(s->stream, &g);
   if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
   }
   if (e == cudaSuccess) e = cudaGraphInstantiate(&s->pexec, g, 0);
   if (g) cudaGraphDestroy(g);
   if (e != cudaSuccess) {
      cudaGetLastError();
      s->prep_ok = -1;
      return 0;
   }
   s->prep_ok = 1;
   return 0;
}

int pgb_vcycle(pgb_solver *s, double *res)
{
   int rc;
   if (s->host_only) return fail(4, "solver was created with PGB_HOST_ONLY");
   if (!s->prepared && (rc = pgb_prepare(s))) return rc;
   if (getenv("PGB_NO_GRAPH")) {
      if ((rc = vcycle_launch(s))) return rc;
      CU(cudaMemcpyAsync(s->h_res, norm_slot(s, s->h.nlev, N_RESID), sizeof(double),
                         cudaMemcpyDeviceToHost, s->stream));
   } else {
      if (!s->graph_ok && (rc = build_graph(s))) return rc;
      CU(cudaGraphLaunch(s->gexec, s->stream));
      g_graph_replayed += s->graph_kernels;
   }
   CU(cudaStreamSynchronize(s->stream));
   *res = s->h_res[0];
   if (s->d_tmaps) {   /* a TMA sweep's wait that timed out leaves a flag */
      int err = 0;
      CU(cudaMemcpy(&err, s->d_err, sizeof(int), cudaMemcpyDeviceToHost));
      if (err) {
         CU(cudaMemset(s->d_err, 0, sizeof(int)));
         return fail(12, "a device wait for staged data timed out (TMA sweep); results are not valid");
      }
   }
   return 0;
}

/* the end of pgb_solve once the stream is idle: the statistics (cycles in
 * it, coarsest iterations and the device-timed error word in h_res) */
static int solve_done(pgb_solver *s, int it, double res, int *iters, double *res_final)
{
   float ms = 0;
   int ci = 0, err = 0;
   CU(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
   memcpy(&ci, s->h_res + 1, sizeof(int));
   memcpy(&err, s->h_res + 3, sizeof(int));
   if (err) {
      CU(cudaMemsetAsync(s->d_err, 0, sizeof(int), s->stream));
      return fail(12, "a device wait for staged data timed out (TMA sweep); results are not valid");
   }
   s->last_cycles = it;
   s->last_citers = ci;
   s->last_ms = ms;
   if (iters) *iters = it;
   if (res_final) *res_final = res;
   return 0;
}

int pgb_solve(pgb_solver *s, int *iters, double *res_final, double *res_per_cycle, int cap)
{
   const pgb_hparams *p = &s->h.prm;
   double res = p->tol + 1;
   int it = 0, rc;
   if (s->host_only) return fail(4, "solver was created with PGB_HOST_ONLY");
   CU(cudaEventRecord(s->ev0, s->stream));
   if (!getenv("PGB_NO_GRAPH") && (p->precision != PGB_MIXED || s->tuned) && !s->prep_ok &&
       (rc = build_prepare_graph(s)))
      return rc;
   if (s->prep_ok > 0 && !getenv("PGB_NO_GRAPH")) {
      CU(cudaGraphLaunch(s->pexec, s->stream));
      s->prepared = 1;
   } else if ((rc = pgb_prepare(s)))
      return rc;
   if (!getenv("PGB_NO_GRAPH") && !getenv("PGB_HOST_LOOP") && p->max_iter > 0) {
      if (!s->graph_ok && (rc = build_graph(s))) return rc;   /* also counts the cycle's kernels */
      if (!s->solve_ok && (rc = build_solve_graph(s))) return rc;
   }
   if (s->solve_ok > 0 && !getenv("PGB_NO_GRAPH") && !getenv("PGB_HOST_LOOP") && p->max_iter > 0) {
      /* one wait for everything: the cycle count, the last norm and the
       * norm history up to cap (entries past the count are not used) */
      const int nh = cap < p->max_iter ? cap : p->max_iter;
      CU(cudaMemsetAsync(s->d_it, 0, sizeof(int), s->stream));
      CU(cudaGraphLaunch(s->sexec, s->stream));
      CU(cudaEventRecord(s->ev1, s->stream));
      CU(cudaMemcpyAsync(s->h_res + 2, s->d_it, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
      CU(cudaMemcpyAsync(s->h_res, norm_slot(s, s->h.nlev, N_RESID), sizeof(double), cudaMemcpyDeviceToHost,
                         s->stream));
      CU(cudaMemcpyAsync(s->h_res + 1, s->d_citers, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
      CU(cudaMemcpyAsync(s->h_res + 3, s->d_err, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
      if (res_per_cycle && nh > 0)
         CU(cudaMemcpyAsync(res_per_cycle, s->d_hist, sizeof(double) * (size_t)nh, cudaMemcpyDeviceToHost,
                            s->stream));
      CU(cudaStreamSynchronize(s->stream));
      memcpy(&it, s->h_res + 2, sizeof(int));
      res = s->h_res[0];
      g_graph_replayed += (s->graph_kernels + 1) * it;
      return solve_done(s, it, res, iters, res_final);
   } else
      while ((it < p->min_iter || res > p->tol) && it < p->max_iter) {
         if ((rc = pgb_vcycle(s, &res))) return rc;
         if (res_per_cycle && it < cap) res_per_cycle[it] = res;
         it++;
      }
   CU(cudaEventRecord(s->ev1, s->stream));
   CU(cudaMemcpyAsync(s->h_res + 1, s->d_citers, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
   CU(cudaMemcpyAsync(s->h_res + 3, s->d_err, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
   CU(cudaStreamSynchronize(s->stream));
   return solve_done(s, it, res, iters, res_final);
}

int pgb_stats(const pgb_solver *s, int *vcycles, long *coarsest_iters, double *device_ms)
{
   if (vcycles) *vcycles = s->last_cycles;
   if (coarsest_iters) *coarsest_iters = s->last_citers;
   if (device_ms) *device_ms = s->last_ms;
   return 0;
}

long long pgb_launch_count(void)
{
   return (long long)(pgb_dev_launches() + pgb_dev_launches32() + pgb_dev_launches_ex() +
                      pgb_dev_launches_net() + pgb_dev_launches_bo() + pgb_dev_launches_diss() +
                      pgb_dev_launches_lb()) - g_captured + g_graph_replayed;
}

int pgb_time_relax(pgb_solver *s, int L, int reps, double *ms_per_sweep, double *bytes_per_sweep)
{
   int r, b;
   float ms = 0;
   double pts = 0;
   if (s->host_only) return fail(4, "solver was created with PGB_HOST_ONLY");
   if (L < 1 || L > s->h.nlev || reps < 1) return fail(3, "bad level or reps");
   int mixed = s->h.prm.precision == PGB_MIXED;
   for (b = 0; b < s->h.lev[L].nbox; b++) pts += s->h.boxes[s->h.lev[L].box[b]].count;
   /* the mixed form's sweeps run as a smoothing block of the V-cycle does
    * (pre_swp sweeps with the level's tuned tile depth and sweeps per
    * launch, no sync between them) */
   int nsw = mixed && s->h.prm.pre_swp > 0 ? s->h.prm.pre_swp : 1;
   if (mixed && !s->tuned && autotune(s)) return 10;
   s->prepared = 0;   /* the sweeps change the level: the next cycle starts from pgb_prepare */
   for (r = 0; r <= reps; r++) {
      if (r == 1) CU(cudaEventRecord(s->ev0, s->stream));   /* first block warms up */
      int slot = PGB_W32_E;
      if (mixed) KC32(pgb_k_sweep32(s->dbox, s->lv[L], nsw, s->fuse[L], &slot, s->stream));
      else if (relax(s, L, N_RELAX_UP)) return 11;
   }
   CU(cudaEventRecord(s->ev1, s->stream));
   CU(cudaEventSynchronize(s->ev1));
   CU(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
   if (ms_per_sweep) *ms_per_sweep = ms / ((double)reps * nsw);
   /* FP64 sweep: u read+write, rhs, src (32 B); FP32 sweep on the
    * correction: e read+write, defect, Jacobian term (16 B) */
   if (bytes_per_sweep) *bytes_per_sweep = (mixed ? 16.0 : 32.0) * pts;
   return 0;
}

/* ------------------------------------------------- AMR-hierarchy transfers -- */
int pgb_amr_interp(pgb_solver *s, int lc, int amr_bdy_width, int order)
{
   pgb_plan p;
   int rc;
   if (s->host_only) return fail(4, "solver was created with PGB_HOST_ONLY");
   if (order != 2 && order != 4) return fail(3, "interpolation order must be 2 or 4");
   if (amr_bdy_width < 0) return fail(3, "AMR boundary width must be >= 0");
   if ((rc = pgb_plan_amr_interp(&s->h, lc, amr_bdy_width, order, &p)) != 0) {
      pgb_plan_release(&p);
      return fail(3, "%s", s->h.err);
   }
   rc = upload_plan(&p, sizeof(pgb_interp_op));
   if (!rc && p.nops) {   /* every elliptic variable */
      int v;
      for (v = 0; v < s->nvar && !rc; v++)
         if (pgb_k_interp(s->dbox, &p, PGB_FV(v, PGB_F_U), s->h.dim, s->stream)) rc = fail(11, "AMR interpolation failed");
      if (!rc && cudaStreamSynchronize(s->stream) != cudaSuccess) rc = fail(11, "AMR interpolation failed");
   }
   free_plan_dev(&p);
   pgb_plan_release(&p);
   s->prepared = 0;   /* u changed */
   return rc;
}

/* Regrid (PAMR_compose_hierarchy's init_new_cgh, src/gh.c:934-1045): u and
 * the sources of every AMR level of dst, a solver built on the hierarchy
 * after a regrid, from src, the solver of the hierarchy it replaces. Level
 * by level, coarse to fine: on levels >= min_level the interpolation from
 * src's next coarser level over the whole new level, then on every level
 * the copies from src's grids of the same level where they overlap (the
 * reference keeps the levels below the recomposed range as they are, which
 * the copies reproduce on unchanged grids). Both transfers read src only.
 * Points of a new level that neither covers keep dst's values. */
int pgb_regrid(pgb_solver *dst, pgb_solver *src, int order, int min_level)
{
   pgb_dbox *joint = 0;
   int rc = 0, Ln, f, namr = 0, l;
   if (dst->host_only || src->host_only) return fail(4, "solver was created with PGB_HOST_ONLY");
   if (dst == src) return fail(3, "regrid: source and destination are the same solver");
   if (order != 2 && order != 4) return fail(3, "interpolation order must be 2 or 4");
   if (dst->h.dim != src->h.dim || dst->nsrc != src->nsrc || dst->nvar != src->nvar)
      return fail(3, "regrid: the solvers differ in dimension, source or variable count");
   if (min_level < 1) return fail(3, "regrid: min_level must be >= 1");
   for (l = 1; l <= dst->h.nlev; l++) namr += dst->h.lev[l].in_amrh ? 1 : 0;
   if (cudaStreamSynchronize(src->stream) != cudaSuccess) return fail(11, "regrid: source stream");
   if (cudaMalloc((void **)&joint, sizeof(pgb_dbox) * (size_t)(src->h.nbox + dst->h.nbox)) != cudaSuccess)
      return fail(10, "regrid: device box table");
   if (cudaMemcpyAsync(joint, src->dbox, sizeof(pgb_dbox) * (size_t)src->h.nbox, cudaMemcpyDeviceToDevice,
                       dst->stream) != cudaSuccess ||
       cudaMemcpyAsync(joint + src->h.nbox, dst->dbox, sizeof(pgb_dbox) * (size_t)dst->h.nbox,
                       cudaMemcpyDeviceToDevice, dst->stream) != cudaSuccess)
      rc = fail(10, "regrid: device box table");
   for (Ln = dst->h.prm.min_level; !rc && Ln < dst->h.prm.min_level + namr; Ln++) {
      pgb_plan pi, pc;
      char err[256];
      if (pgb_plan_regrid(&src->h, &dst->h, Ln, order, Ln >= min_level, &pi, &pc, err, sizeof(err))) {
         rc = fail(3, "regrid: %s", err);
      } else if (upload_plan(&pi, sizeof(pgb_interp_op)) || upload_plan(&pc, sizeof(pgb_copy_op))) {
         rc = fail(10, "regrid: plan upload");
      } else {
         /* the fields the AMR hierarchy carries: every elliptic variable and every source */
         for (f = 0; f < dst->nvar + dst->nsrc && !rc; f++) {
            const int field = f < dst->nvar ? PGB_FV(f, PGB_F_U) : PGB_SRC_FIELD(f - dst->nvar);
            if ((pi.nops && pgb_k_interp(joint, &pi, field, dst->h.dim, dst->stream)) ||
                (pc.nops && pgb_k_copy(joint, &pc, field, dst->stream)))
               rc = fail(11, "regrid: transfer kernels failed");
         }
         if (!rc && cudaStreamSynchronize(dst->stream) != cudaSuccess) rc = fail(11, "regrid: transfer failed");
      }
      free_plan_dev(&pi);
      free_plan_dev(&pc);
      pgb_plan_release(&pi);
      pgb_plan_release(&pc);
   }
   cudaStreamSynchronize(dst->stream);
   cudaFree(joint);
   dst->prepared = 0;   /* u and the sources changed */
   return rc;
}

/* ------------------------------------------------------------ checkpoint -- */
/* File layout (little-endian as written by the host): "PGBCKPT1", int32
 * version, dim, operator kind, ngrids, source count, elliptic variables,
 * then a 64-bit hash of the variables' operator programs; per input grid
 * int32 level, shape[3], double bbox[6], then u of each variable and each
 * source (float64, x fastest). Version 2 files (one variable, 0 in the
 * variables' slot) load as well. Grids below the hierarchy's coarsest AMR
 * level are not part of it and are skipped. */
#define CKPT_MAGIC "PGBCKPT1"
#define CKPT_VERSION 3

static unsigned long long dop_hash(const pgb_dop *d)
{
   const unsigned char *p = (const unsigned char *)d;
   unsigned long long h = 1469598103934665603ull;
   size_t i;
   for (i = 0; i < sizeof(*d); i++) h = (h ^ p[i]) * 1099511628211ull;
   return h;
}

/* the operators of all variables (one variable: the hash of its operator) */
static unsigned long long ops_hash(const pgb_solver *s)
{
   unsigned long long h = dop_hash(&s->dop);
   int v;
   for (v = 1; v < s->nvar; v++) h = h * 1099511628211ull ^ dop_hash(&s->dops[v]);
   return h;
}

int pgb_checkpoint_save(pgb_solver *s, const char *path)
{
   FILE *f;
   int g, rc = 0;
   const int hdr[6] = {CKPT_VERSION, s->h.dim, s->h.pde, s->h.ngrids, s->nsrc, s->nvar};
   const unsigned long long oh = ops_hash(s);
   if (s->host_only) return fail(4, "solver was created with PGB_HOST_ONLY");
   if (!(f = fopen(path, "wb"))) return fail(5, "checkpoint: cannot open %s for writing", path);
   if (fwrite(CKPT_MAGIC, 1, 8, f) != 8 || fwrite(hdr, sizeof(int), 6, f) != 6 || fwrite(&oh, 8, 1, f) != 1)
      rc = fail(5, "checkpoint: write failed");
   for (g = 0; g < s->h.ngrids && !rc; g++) {
      if (s->h.grid_box[g] < 0) continue;
      const pgb_hbox *b = &s->h.boxes[s->h.grid_box[g]];
      const pgb_dbox *db = &s->hbox[s->h.grid_box[g]];
      const size_t n = (size_t)b->shape[0] * b->shape[1] * b->shape[2];
      const int meta[4] = {b->level, b->shape[0], b->shape[1], b->shape[2]};
      double *buf = (double *)malloc(sizeof(double) * n);
      int k;
      if (!buf) {
         rc = fail(10, "checkpoint: host buffer");
         break;
      }
      if (fwrite(meta, sizeof(int), 4, f) != 4 || fwrite(b->bbox, sizeof(double), 6, f) != 6)
         rc = fail(5, "checkpoint: write failed");
      for (k = 0; k < s->nvar + s->nsrc && !rc; k++) {   /* u of each variable, then the sources */
         if (cudaMemcpyAsync(buf, db->f[k >= s->nvar ? PGB_SRC_FIELD(k - s->nvar) : PGB_FV(k, PGB_F_U)],
                             sizeof(double) * n, cudaMemcpyDeviceToHost, s->stream) != cudaSuccess ||
             cudaStreamSynchronize(s->stream) != cudaSuccess)
            rc = fail(11, "checkpoint: device read failed");
         else if (fwrite(buf, sizeof(double), n, f) != n)
            rc = fail(5, "checkpoint: write failed");
      }
      free(buf);
   }
   if (fclose(f) && !rc) rc = fail(5, "checkpoint: close failed");
   return rc;
}

/* Reads and checks the whole file before anything is copied to the device;
 * a copy that then fails (a CUDA error) can leave earlier grids restored. */
int pgb_checkpoint_load(pgb_solver *s, const char *path)
{
   FILE *f;
   char magic[8];
   int hdr[6], g, k, rc = 0, ng = s->h.ngrids;
   const int nf = s->nsrc + s->nvar;
   unsigned long long oh = 0;
   double **buf;
   if (s->host_only) return fail(4, "solver was created with PGB_HOST_ONLY");
   if (!(f = fopen(path, "rb"))) return fail(5, "checkpoint: cannot open %s", path);
   if (fread(magic, 1, 8, f) != 8 || memcmp(magic, CKPT_MAGIC, 8) || fread(hdr, sizeof(int), 6, f) != 6 ||
       fread(&oh, 8, 1, f) != 1) {
      fclose(f);
      return fail(6, "checkpoint: %s is not a checkpoint", path);
   }
   if (!(hdr[0] == CKPT_VERSION || (hdr[0] == 2 && hdr[5] == 0)) || hdr[1] != s->h.dim || hdr[2] != s->h.pde ||
       hdr[3] != ng || hdr[4] != s->nsrc || (hdr[0] == 2 ? 1 : hdr[5]) != s->nvar || oh != ops_hash(s)) {
      fclose(f);
      return fail(6, "checkpoint: version, dimension, operators, variable or grid count differ from the solver's");
   }
   buf = (double **)calloc((size_t)nf * (size_t)(ng ? ng : 1), sizeof(double *));
   if (!buf) {
      fclose(f);
      return fail(10, "checkpoint: host buffer");
   }
   for (g = 0; g < ng && !rc; g++) {
      if (s->h.grid_box[g] < 0) continue;
      const pgb_hbox *b = &s->h.boxes[s->h.grid_box[g]];
      const size_t n = (size_t)b->shape[0] * b->shape[1] * b->shape[2];
      int meta[4];
      double bb[6];
      if (fread(meta, sizeof(int), 4, f) != 4 || fread(bb, sizeof(double), 6, f) != 6) {
         rc = fail(6, "checkpoint: truncated");
         break;
      }
      if (meta[0] != b->level || meta[1] != b->shape[0] || meta[2] != b->shape[1] || meta[3] != b->shape[2] ||
          memcmp(bb, b->bbox, sizeof(bb))) {
         rc = fail(6, "checkpoint: grid %d differs from the solver's hierarchy", g);
         break;
      }
      for (k = 0; k < nf && !rc; k++) {
         double *v = (double *)malloc(sizeof(double) * n);
         buf[(size_t)nf * g + k] = v;
         if (!v) rc = fail(10, "checkpoint: host buffer");
         else if (fread(v, sizeof(double), n, f) != n) rc = fail(6, "checkpoint: truncated");
      }
   }
   fclose(f);
   for (g = 0; g < ng && !rc; g++) {
      if (s->h.grid_box[g] < 0) continue;
      const size_t o = (size_t)nf * g;
      rc = pgb_set_grid(s, g, buf[o], buf[o + s->nvar]);
      for (k = 1; k < s->nvar && !rc; k++) rc = pgb_set_var(s, g, k, buf[o + k]);
      for (k = 1; k < s->nsrc && !rc; k++) rc = pgb_set_source(s, g, k, buf[o + s->nvar + k]);
   }
   for (g = 0; g < nf * ng; g++) free(buf[g]);
   free(buf);
   return rc;
}

/* ---------------------------------------------------------------- trace -- */
int pgb_trace_enable(pgb_solver *s, int capacity)
{
   int hdr[4] = {0, capacity, 0, 0};
   if (s->host_only) return fail(4, "solver was created with PGB_HOST_ONLY");
   drop_graph(s);   /* the trace pointer is baked into the captured launches */
   if (s->d_trace) cudaFree(s->d_trace);
   s->d_trace = 0;
   s->trace_cap = 0;
   if (capacity <= 0) return 0;
   CU(cudaMalloc((void **)&s->d_trace, sizeof(pgb_trace) + sizeof(pgb_trace_rec) * (size_t)capacity));
   CU(cudaMemcpy(s->d_trace, hdr, sizeof(hdr), cudaMemcpyHostToDevice));
   s->trace_cap = capacity;
   return 0;
}

int pgb_trace_fetch(pgb_solver *s, int *kind, int *level, int *box, int *repeat, double *norm,
                    int cap, int *n)
{
   int hdr[4], i, m;
   pgb_trace_rec *r;
   if (!s->d_trace) return fail(5, "trace not enabled");
   CU(cudaStreamSynchronize(s->stream));
   CU(cudaMemcpy(hdr, s->d_trace, sizeof(hdr), cudaMemcpyDeviceToHost));
   m = hdr[0] < cap ? hdr[0] : cap;
   r = (pgb_trace_rec *)malloc(sizeof(pgb_trace_rec) * (size_t)(m ? m : 1));
   CU(cudaMemcpy(r, s->d_trace->rec, sizeof(pgb_trace_rec) * (size_t)m, cudaMemcpyDeviceToHost));
   for (i = 0; i < m; i++) {
      kind[i] = r[i].kind;
      level[i] = r[i].level;
      box[i] = r[i].box;
      repeat[i] = r[i].repeat;
      norm[i] = r[i].norm;
   }
   free(r);
   *n = m;
   hdr[0] = 0;
   CU(cudaMemcpy(s->d_trace, hdr, sizeof(int), cudaMemcpyHostToDevice));
   if (hdr[2]) return fail(6, "trace overflowed");
   return 0;
}

/* ------------------------------------------------------------ queries -- */
int pgb_num_levels(const pgb_solver *s) { return s->h.nlev; }

int pgb_level_nbox(const pgb_solver *s, int L)
{
   if (L < 1 || L > s->h.nlev) return -1;
   return s->h.lev[L].nbox;
}

static const pgb_hbox *lbox(const pgb_solver *s, int L, int idx)
{
   if (L < 1 || L > s->h.nlev || idx < 0 || idx >= s->h.lev[L].nbox) return 0;
   return &s->h.boxes[s->h.lev[L].box[idx]];
}

int pgb_box_info(const pgb_solver *s, int L, int idx, int *shape3, double *bbox6, int *coarsest,
                 int *amr_grid)
{
   const pgb_hbox *b = lbox(s, L, idx);
   if (!b) return fail(3, "no box %d on level %d", idx, L);
   if (shape3) memcpy(shape3, b->shape, sizeof(int) * 3);
   if (bbox6) memcpy(bbox6, b->bbox, sizeof(double) * 6);
   if (coarsest) *coarsest = b->coarsest;
   if (amr_grid) *amr_grid = b->amr_grid;
   return 0;
}

int pgb_box_cmask(const pgb_solver *s, int L, int idx, int kind, double *out)
{
   const pgb_hbox *b = lbox(s, L, idx);
   long n, i;
   const uint8_t *m;
   if (!b) return fail(3, "no box %d on level %d", idx, L);
   m = kind ? b->child_mask : b->bdy_mask;
   n = (long)b->shape[0] * b->shape[1] * b->shape[2];
   for (i = 0; i < n; i++) out[i] = m[i] ? 1.0 : 0.0;
   return 0;
}

static int level_index(const pgb_solver *s, int box)
{
   const pgb_hlevel *lv = &s->h.lev[s->h.boxes[box].level];
   int i;
   for (i = 0; i < lv->nbox; i++)
      if (lv->box[i] == box) return i;
   return -1;
}

int pgb_plan_dump(const pgb_solver *s, int which, int L, int *rows, int cap)
{
   const pgb_plan *p;
   int i;
   if (L < 1 || L > s->h.nlev) return -fail(3, "level %d out of range", L);
   switch (which) {
   case 0: p = &s->h.sync[L][0]; break;
   case 1: p = &s->h.sync[L][1]; break;
   case 2: p = &s->h.sync_coarsest[L]; break;
   case 3: p = &s->h.inject[L]; break;
   case 4: p = &s->h.inject_init[L]; break;
   case 5: p = &s->h.interp[L]; break;
   default: return -fail(3, "unknown plan %d", which);
   }
   for (i = 0; i < p->nops && i < cap; i++) {
      int *r = rows + 24 * i, sb, db;
      memset(r, 0, sizeof(int) * 24);
      if (which <= 2) {
         const pgb_copy_op *o = (const pgb_copy_op *)p->h_ops + i;
         sb = o->src_box; db = o->dst_box;
         r[4] = o->i1; r[5] = o->j1; r[6] = o->k1; r[7] = o->i2; r[8] = o->j2; r[9] = o->k2;
         r[10] = o->ni; r[11] = o->nj; r[12] = o->nk;
      } else if (which <= 4) {
         const pgb_restrict_op *o = (const pgb_restrict_op *)p->h_ops + i;
         int f;
         sb = o->src_box; db = o->dst_box;
         r[4] = o->i1; r[5] = o->j1; r[6] = o->k1; r[7] = o->i2; r[8] = o->j2; r[9] = o->k2;
         r[10] = o->ni; r[11] = o->nj; r[12] = o->nk; r[13] = o->irho;
         for (f = 0; f < PGB_F_VAR1; f++) r[14 + f] = o->op[f];   /* variable 0 and the sources */
      } else {
         const pgb_interp_op *o = (const pgb_interp_op *)p->h_ops + i;
         sb = o->src_box; db = o->dst_box;
         r[4] = o->i1i; r[5] = o->j1i; r[6] = o->k1i; r[7] = o->nii; r[8] = o->nji; r[9] = o->nki;
         r[10] = o->i2b; r[11] = o->j2b; r[12] = o->k2b; r[13] = o->i2; r[14] = o->j2; r[15] = o->k2;
         r[16] = o->nib; r[17] = o->njb; r[18] = o->nkb; r[19] = o->irho; r[20] = o->ord;
      }
      r[0] = s->h.boxes[sb].level;
      r[1] = level_index(s, sb);
      r[2] = s->h.boxes[db].level;
      r[3] = level_index(s, db);
   }
   return p->nops;
}
