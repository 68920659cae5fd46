/*
 * libamrd_mg_gb300: AMRD's multigrid module (amrd/mg.c) as a drop-in that
 * solves on the GPU through libpamr_gb300 (interface in amrd_mg_gb300.h).
 *
 * Data flow of solve_elliptics(L, tl, save_tre) (amrd/mg.c:20-79):
 *   1. the hierarchy of AMR levels L..Lf is read through PAMR: the
 *      sequential grids of each level in the order the application composed
 *      them (PAMR_get_sgh, which build_mgh's island coarsening depends on,
 *      src/gh.c:1285-1300), the global bbox and level-1 spacing;
 *   2. libpamr_gb300 builds the same MG hierarchy and transfer plans once
 *      and keeps them while the AMR hierarchy and parameters are unchanged
 *      (the reference rebuilds both on every solve);
 *   3. the elliptic variable and the operator's sources at time level tl
 *      are copied from PAMR's grids (PAMR_get_g_attribs) to the device, the
 *      V-cycles run there, the solution is copied back into the same PAMR
 *      arrays, and the AMR cmask of levels L..Lf gets the boundary mask the
 *      reference's last set_cmask_bdy leaves in it (amrd/mg.c:132, the MG
 *      cmask aliases the AMR one, src/gh.c:1139-1147).
 * vcycle(giter, save_tre) (amrd/mg.c:84-201) works on the MG hierarchy the
 * caller built with PAMR_build_mgh: every elliptic variable's u and the
 * sources of every MG level are copied from PAMR's MG grids (PAMR built or
 * injected them there), one V-cycle runs on the device, and each variable's
 * u on every MG level, its f_res on the finest and the sources the cycle
 * injected into the pure MG levels come back.
 *
 * Limits (each reported by a message and AMRD_stop, as AMRD reports
 * errors): up to four elliptic variables (FP64 form, every variable with
 * the first one's MG transfers);
 * save_tre = 0; no periodic boundaries;
 * no t0 initialisation hook or constraint-data variables (AMRD_is_t0 runs
 * of generate_id with app_elliptic_vars_t0_init / MG_cnst_data); one MPI
 * rank; mg_sync and mg_interp2 set on the variable (the reference
 * without them skips the sync or the correction, which the device plans do
 * not model); equal min_mg_cwidth in every dimension.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "amrd_abi.h"
#include "amrd_mg_gb300.h"
#include "pamr_gb300.h"

#define MAXSRC PGB_MAX_SOURCES

static struct {
   /* registration */
   pgb_operator *op;
   pgb_operator *var_op[PGB_MAX_VARS];   /* elliptic variables 1.. (var_op[0] unused) */
   char *src_names[MAXSRC];
   int nsrc;
   int precision;
   int op_generation;
   /* the cached device hierarchy and what it was built from */
   pgb_solver *s;
   int dim, L, ngrids, generation, nvar;
   int *lev;
   double *bbox;            /* 6 per grid */
   pgb_mg_params prm;
   int restr_src[MAXSRC];
   int base_shape[3];
   double base_bbox[6];
   /* per input grid: MG level and box index (for the cmask write-back) */
   int *mg_level, *mg_idx;
   /* residual history of the last solve */
   double *hist;
   int nhist;
} G;

static void stop(const char *what, const char *detail)
{
   char a[512], b[512];
   snprintf(a, sizeof(a), "libamrd_mg_gb300: %s", what);
   snprintf(b, sizeof(b), "%s", detail ? detail : "");
   AMRD_stop(a, b);
}

static int ok_pgb(int rc, const char *what)
{
   if (rc) {
      fprintf(stderr, "libamrd_mg_gb300: %s: %s\n", what, pgb_last_error());
      stop(what, pgb_last_error());
   }
   return rc == 0;
}

/* ------------------------------------------------------------ registration -- */
int amrd_set_device_MG_operator(int nsrc, char **src_names, char *lop, char *jac)
{
   pgb_operator *op = 0;
   int k;
   if (nsrc < 0 || nsrc > MAXSRC) {
      printf("amrd_set_device_MG_operator: error ... %d sources (at most %d)\n", nsrc, MAXSRC);
      return 0;
   }
   if (pgb_operator_create(nsrc, lop, jac, &op)) {
      printf("amrd_set_device_MG_operator: error ... %s\n", pgb_last_error());
      return 0;
   }
   for (k = 0; k < nsrc; k++)
      if (!src_names || !src_names[k]) {
         printf("amrd_set_device_MG_operator: error ... source %d has no name\n", k);
         pgb_operator_destroy(op);
         return 0;
      }
   if (G.op) pgb_operator_destroy(G.op);
   for (k = 0; k < MAXSRC; k++) {
      free(G.src_names[k]);
      G.src_names[k] = k < nsrc ? strdup(src_names[k]) : 0;
   }
   G.op = op;
   G.nsrc = nsrc;
   G.op_generation++;
   return 1;
}

int amrd_set_device_MG_var_operator(int var, char *lop, char *jac)
{
   pgb_operator *op = 0;
   if (var < 1 || var >= PGB_MAX_VARS) {
      printf("amrd_set_device_MG_var_operator: error ... variable %d (1..%d)\n", var, PGB_MAX_VARS - 1);
      return 0;
   }
   if (!G.op) {
      printf("amrd_set_device_MG_var_operator: error ... register variable 0 (amrd_set_device_MG_operator) first\n");
      return 0;
   }
   if (pgb_operator_create(G.nsrc, lop, jac, &op)) {
      printf("amrd_set_device_MG_var_operator: error ... %s\n", pgb_last_error());
      return 0;
   }
   if (G.var_op[var]) pgb_operator_destroy(G.var_op[var]);
   G.var_op[var] = op;
   G.op_generation++;
   return 1;
}

int amrd_set_device_MG_precision(int precision)
{
   if (precision != PGB_FP64 && precision != PGB_MIXED) {
      printf("amrd_set_device_MG_precision: error ... precision must be 0 or 1\n");
      return 0;
   }
   G.precision = precision;
   return 1;
}

int amrd_device_MG_residuals(double *res, int cap)
{
   int i;
   for (i = 0; i < G.nhist && i < cap; i++) res[i] = G.hist[i];
   return G.nhist;
}

static void release(void)
{
   if (G.s) pgb_destroy(G.s);
   G.s = 0;
   free(G.lev);
   free(G.bbox);
   free(G.mg_level);
   free(G.mg_idx);
   G.lev = 0;
   G.bbox = 0;
   G.mg_level = G.mg_idx = 0;
   G.ngrids = 0;
}

void amrd_device_MG_release(void) { release(); }

/* ---------------------------------------------------------- PAMR queries -- */
typedef struct {
   int rank, dim, shape[3], gw[6], ngfs, level;
   double bbox[6], t, *x[3], **gfs;
} pgrid;

static double *g_gfs[4096];   /* PAMR_get_g_attribs fills one pointer per gfn */

static int attribs(pgrid *g)
{
   int d;
   g->shape[0] = g->shape[1] = g->shape[2] = 1;
   memset(g->bbox, 0, sizeof(g->bbox));
   g->gfs = g_gfs;
   if (!PAMR_get_g_attribs(&g->rank, &g->dim, g->shape, g->bbox, g->gw, &g->t, &g->ngfs, g->x, g->gfs))
      return 0;
   for (d = g->dim; d < 3; d++) g->shape[d] = 1;
   return 1;
}

static int same_bbox(const double *a, const double *b, int dim, const double *dx)
{
   int i;
   for (i = 0; i < 2 * dim; i++)
      if (fabs(a[i] - b[i]) > 0.25 * dx[i / 2]) return 0;
   return 1;
}

/* mg_inject / mg_interp / mg_sync / in_mgh / num_tl / mg_noinj_to_amr of a variable */
typedef struct {
   int in_amrh, in_mgh, num_tl, mg_inject, mg_interp, mg_sync, mg_noinj_to_amr;
} vattr;

static int var_attr(const char *name, vattr *a)
{
   int amr_inject, amr_interp, amr_bdy_interp, amr_sync, regrid, pbt[2 * ABI_PAMR_MAX_DIM];
   return PAMR_get_var_attribs((char *)name, &a->in_amrh, &a->in_mgh, &a->num_tl, &amr_inject, &amr_interp,
                               &amr_bdy_interp, &amr_sync, &a->mg_inject, &a->mg_interp, &a->mg_sync,
                               &a->mg_noinj_to_amr, &regrid, pbt);
}

/* MG parameters from AMRD's globals and the variables' transfer bits
 * (amrd/io.c:855-871: f_res carries the restriction of the residual and the
 * interpolation order of the coarse-grid correction) */
static void read_params(pgb_mg_params *p, int *restr_src)
{
   const char *var = AMRD_elliptic_vars[0];
   char res_name[512];
   vattr a, ar;
   int cw[ABI_PAMR_MAX_DIM] = {0, 0, 0}, per[ABI_PAMR_MAX_DIM] = {0, 0, 0}, ib = 2, d, k, dim = 0;
   double bb[6];
   pgb_default_params(p);
   p->pre_swp = AMRD_MG_pre_swp;
   p->pst_swp = AMRD_MG_pst_swp;
   p->max_iter = AMRD_MG_max_iter;
   p->min_iter = AMRD_MG_min_iter;
   p->max_citer = AMRD_MG_max_citer;
   p->tol = AMRD_MG_tol;
   p->crtol = AMRD_MG_crtol;
   p->w0_r = AMRD_MG_w0_r;
   p->w0_i = AMRD_MG_w0_i;
   p->precision = G.precision;
   snprintf(res_name, sizeof(res_name), "%s_res", var);
   if (!var_attr(var, &a) || !var_attr(res_name, &ar)) stop("cannot read the elliptic variable's attributes", var);
   if (a.mg_sync != 1) stop("the elliptic variable must be in mg_sync", var);
   if (ar.mg_interp != 2 && ar.mg_interp != 4) stop("the elliptic variable must be in mg_interp2", var);
   if (a.mg_noinj_to_amr) stop("the elliptic variable must be injected to AMR levels", var);
   p->restr_u = a.mg_inject;
   p->restr_res = ar.mg_inject;
   p->interp_order = ar.mg_interp;
   for (k = 1; k < AMRD_num_elliptic_vars; k++) {   /* the others take the same transfers */
      vattr b, br;
      const char *vk = AMRD_elliptic_vars[k];
      snprintf(res_name, sizeof(res_name), "%s_res", vk);
      if (!var_attr(vk, &b) || !var_attr(res_name, &br)) stop("cannot read an elliptic variable's attributes", vk);
      if (b.mg_sync != a.mg_sync || b.mg_inject != a.mg_inject || b.mg_noinj_to_amr != a.mg_noinj_to_amr ||
          br.mg_inject != ar.mg_inject || br.mg_interp != ar.mg_interp)
         stop("every elliptic variable must take the first one's MG transfers on the device", vk);
   }
   for (k = 0; k < G.nsrc; k++) {
      vattr s;
      if (!var_attr(G.src_names[k], &s)) stop("unknown source variable", G.src_names[k]);
      if (!s.in_amrh || !s.in_mgh) stop("a source must live in both hierarchies", G.src_names[k]);
      if (!s.mg_noinj_to_amr) stop("a source must not be injected back to AMR levels", G.src_names[k]);
      restr_src[k] = s.mg_inject;
   }
   p->restr_src = G.nsrc ? restr_src[0] : PGB_HW_RESTR;
   PAMR_get_MG_coarse_width(cw);
   PAMR_get_interp_buffer(&ib);
   PAMR_get_periodic_bdy(per);
   PAMR_get_global_bbox(bb);
   for (d = 0; d < ABI_PAMR_MAX_DIM; d++)
      if (cw[d] > 0) dim = d + 1;
   for (d = 0; d < dim; d++) {
      if (cw[d] != cw[0]) stop("min_mg_cwidth must be the same in every dimension", "");
      if (per[d]) stop("periodic boundaries are not supported on the device", "");
   }
   p->min_cwidth = cw[0];
   p->interp_buffer = ib;
}

/* the sequential grids of AMR levels L..Lf (PAMR_get_sgh), 6 doubles each */
static int read_sgh(int L, int Lf, int dim, int **lev, double **bbox)
{
   int l, n = 0, cap = 0, i, d;
   double *tmp;
   *lev = 0;
   *bbox = 0;
   for (l = L; l <= Lf; l++) {
      int num = 0, valid = PAMR_init_s_iter(l, ABI_PAMR_AMRH, 1);
      while (valid) {
         num++;
         valid = PAMR_next_g();
      }
      cap += num + 8;
   }
   *lev = (int *)malloc(sizeof(int) * (size_t)cap);
   *bbox = (double *)calloc((size_t)cap * 6, sizeof(double));
   tmp = (double *)malloc(sizeof(double) * 2 * ABI_PAMR_MAX_DIM * (size_t)cap);
   for (l = L; l <= Lf; l++) {
      int num = cap - n;
      if (!PAMR_get_sgh(tmp, &num, l)) stop("PAMR_get_sgh failed", "");
      for (i = 0; i < num; i++, n++) {
         (*lev)[n] = l;
         for (d = 0; d < 2 * dim; d++) (*bbox)[6 * n + d] = tmp[2 * dim * i + d];
      }
   }
   free(tmp);
   return n;
}

/* ------------------------------------------------- the device hierarchy -- */
/* (Re)builds the device hierarchy for AMR levels L..Lf unless the cached
 * one was made from the same grids, parameters and operator. */
static void ensure_solver(int L, int Lf)
{
   pgb_mg_params p;
   int restr[MAXSRC] = {PGB_HW_RESTR, PGB_HW_RESTR, PGB_HW_RESTR, PGB_HW_RESTR};
   int *lev, n, d, dim = 0, shape[3] = {1, 1, 1}, i;
   double *bbox, gbb[6] = {0, 0, 0, 0, 0, 0}, dx[3] = {1, 1, 1}, dt;
   pgrid g;
   if (!G.op) stop("no device operator registered (amrd_set_device_MG_operator)", "");
   if (AMRD_num_elliptic_vars < 1 || AMRD_num_elliptic_vars > PGB_MAX_VARS)
      stop("the device solves 1 to 4 elliptic variables", "");
   for (i = 1; i < AMRD_num_elliptic_vars; i++)
      if (!G.var_op[i]) stop("no device operator for an elliptic variable (amrd_set_device_MG_var_operator)",
                             AMRD_elliptic_vars[i]);
   read_params(&p, restr);
   /* dimension and base shape from a level-1 grid's context */
   if (!PAMR_init_s_iter(1, ABI_PAMR_AMRH, 1) || !attribs(&g)) stop("no AMR hierarchy", "");
   dim = g.dim;
   PAMR_get_global_bbox(gbb);
   PAMR_get_dxdt(1, dx, &dt);
   for (d = 0; d < dim; d++) shape[d] = (int)floor((gbb[2 * d + 1] - gbb[2 * d]) / dx[d] + 0.5) + 1;
   n = read_sgh(L, Lf, dim, &lev, &bbox);
   if (G.s && G.dim == dim && G.L == L && G.ngrids == n && G.generation == G.op_generation &&
       G.nvar == AMRD_num_elliptic_vars &&
       !memcmp(G.lev, lev, sizeof(int) * (size_t)n) && !memcmp(G.bbox, bbox, sizeof(double) * 6 * (size_t)n) &&
       !memcmp(&G.prm, &p, sizeof(p)) && !memcmp(G.restr_src, restr, sizeof(restr)) &&
       !memcmp(G.base_shape, shape, sizeof(shape)) && !memcmp(G.base_bbox, gbb, sizeof(gbb))) {
      free(lev);
      free(bbox);
      return;
   }
   release();
   {
      pgb_create_args a;
      pgb_default_create_args(&a);
      a.dim = dim;
      a.op = G.op;
      memcpy(a.base_shape, shape, sizeof(shape));
      memcpy(a.base_bbox, gbb, sizeof(gbb));
      a.ngrids = n;
      a.grid_level = lev;
      a.grid_bbox = bbox;
      a.params = p;
      a.min_level = L;
      for (i = 1; i < MAXSRC; i++) a.restr_src[i] = restr[i];
      a.nvar = AMRD_num_elliptic_vars;
      for (i = 1; i < a.nvar; i++) a.var_op[i] = G.var_op[i];
      if (!ok_pgb(pgb_create_ex(&a, &G.s), "building the device hierarchy")) return;
   }
   G.dim = dim;
   G.L = L;
   G.nvar = AMRD_num_elliptic_vars;
   G.ngrids = n;
   G.lev = lev;
   G.bbox = bbox;
   G.prm = p;
   memcpy(G.restr_src, restr, sizeof(restr));
   memcpy(G.base_shape, shape, sizeof(shape));
   memcpy(G.base_bbox, gbb, sizeof(gbb));
   G.generation = G.op_generation;
   /* input grid -> (MG level, box) */
   G.mg_level = (int *)malloc(sizeof(int) * (size_t)n);
   G.mg_idx = (int *)malloc(sizeof(int) * (size_t)n);
   for (i = 0; i < n; i++) G.mg_level[i] = G.mg_idx[i] = -1;
   for (d = 1; d <= pgb_num_levels(G.s); d++)
      for (i = 0; i < pgb_level_nbox(G.s, d); i++) {
         int ag = -1;
         pgb_box_info(G.s, d, i, 0, 0, 0, &ag);
         if (ag >= 0 && ag < n) {
            G.mg_level[ag] = d;
            G.mg_idx[ag] = i;
         }
      }
}

/* the input grid (sgh entry) a PAMR grid of level l is */
static int grid_index(int l, const pgrid *g)
{
   int i;
   double dx[3] = {1, 1, 1};
   for (i = 0; i < g->dim; i++) dx[i] = g->x[i][1] - g->x[i][0];
   for (i = 0; i < G.ngrids; i++)
      if (G.lev[i] == l && same_bbox(G.bbox + 6 * i, g->bbox, g->dim, dx)) return i;
   return -1;
}

static int gfn(const char *name, int hier, int tl)
{
   int n = PAMR_get_gfn((char *)name, hier, tl);
   if (n < 1) stop("unknown grid function", name);
   return n;
}

/* the AMR time level of a variable's storage that its MG instance uses
 * when the MG hierarchy is built at time level tl (amr_to_mgh,
 * src/gh.c:1139-1147: min(tl, the variable's number of time levels)) */
static int var_tl(const char *name, int tl)
{
   vattr a;
   if (!var_attr(name, &a)) stop("unknown variable", name);
   return tl < a.num_tl ? tl : a.num_tl;
}

/* writes the boundary cmask of box (mg level, idx) into dst */
static void put_bdy_mask(int level, int idx, double *dst)
{
   ok_pgb(pgb_box_cmask(G.s, level, idx, 0, dst), "reading a cmask");
}

/* ------------------------------------------------------------ solve -- */
void solve_elliptics(int L, int tl, int save_tre)
{
   int Lf = PAMR_get_max_lev(ABI_PAMR_AMRH), l, k, iters = 0, cap;
   double res = 0;
   const char *var;
   int gu, gs[MAXSRC], gcm = 0, gv[PGB_MAX_VARS], v;

   if ((AMRD_num_elliptic_vars == 0 && !AMRD_is_t0) ||
       (AMRD_num_elliptic_vars == 0 && AMRD_num_elliptic_vars_t0 == 0 && AMRD_is_t0))
      return;
   if (save_tre) stop("solve_elliptics: save_tre is not supported on the device", "");
   if (AMRD_is_t0 && (app_elliptic_vars_t0_init || AMRD_num_MG_cnst_data_vars > 0))
      stop("solve_elliptics: t0 initialisation hooks are not supported on the device", "");
   ensure_solver(L, Lf);
   var = AMRD_elliptic_vars[0];
   gu = gfn(var, ABI_PAMR_AMRH, var_tl(var, tl));
   for (v = 1; v < G.nvar; v++)
      gv[v] = gfn(AMRD_elliptic_vars[v], ABI_PAMR_AMRH, var_tl(AMRD_elliptic_vars[v], tl));
   for (k = 0; k < G.nsrc; k++) gs[k] = gfn(G.src_names[k], ABI_PAMR_AMRH, var_tl(G.src_names[k], tl));
   if (AMRD_cmask_gfn > 0) gcm = AMRD_cmask_gfn;
   /* copy in */
   for (l = L; l <= Lf; l++) {
      int valid = PAMR_init_s_iter(l, ABI_PAMR_AMRH, 0);
      while (valid) {
         pgrid g;
         int i, sh[3];
         if (!attribs(&g)) stop("PAMR_get_g_attribs failed", "");
         if ((i = grid_index(l, &g)) < 0) stop("a grid of the AMR hierarchy is not in its sequential list", "");
         pgb_grid_shape(G.s, i, sh);
         if (sh[0] != g.shape[0] || sh[1] != g.shape[1] || sh[2] != g.shape[2])
            stop("grid shapes differ from the device hierarchy's", "");
         ok_pgb(pgb_set_grid(G.s, i, g.gfs[gu - 1], G.nsrc ? g.gfs[gs[0] - 1] : 0), "copying a grid");
         for (k = 1; k < G.nsrc; k++) ok_pgb(pgb_set_source(G.s, i, k, g.gfs[gs[k] - 1]), "copying a source");
         for (v = 1; v < G.nvar; v++) ok_pgb(pgb_set_var(G.s, i, v, g.gfs[gv[v] - 1]), "copying a variable");
         valid = PAMR_next_g();
      }
   }
   cap = G.prm.max_iter > 0 ? G.prm.max_iter : 1;
   free(G.hist);
   G.hist = (double *)calloc((size_t)cap, sizeof(double));
   ok_pgb(pgb_solve(G.s, &iters, &res, G.hist, cap), "solve");
   G.nhist = iters;
   AMRD_curr_MG_iter = iters;
   if (AMRD_MG_trace > 1 && my_rank == 0)
      for (k = 0; k < iters; k++) printf("iter %i\t\tres(Lf)=%12.8e\n", k + 1, G.hist[k]);
   /* copy out: u, and the boundary cmask the reference's last V-cycle leaves */
   for (l = L; l <= Lf; l++) {
      int valid = PAMR_init_s_iter(l, ABI_PAMR_AMRH, 0);
      while (valid) {
         pgrid g;
         int i;
         attribs(&g);
         i = grid_index(l, &g);
         ok_pgb(pgb_get_grid(G.s, i, g.gfs[gu - 1]), "reading a grid back");
         for (v = 1; v < G.nvar; v++) ok_pgb(pgb_get_var(G.s, i, v, g.gfs[gv[v] - 1]), "reading a variable back");
         if (gcm && iters > 0) put_bdy_mask(G.mg_level[i], G.mg_idx[i], g.gfs[gcm - 1]);
         valid = PAMR_next_g();
      }
   }
   if (iters == G.prm.max_iter && my_rank == 0 && res > AMRD_MG_tol)
      printf("\nWARNING ... failed to solve elliptics to within %12.8e in %i iterations; res=%12.8e\n",
             AMRD_MG_tol, G.prm.max_iter, res);
   else if (AMRD_MG_trace && my_rank == 0)
      printf("  iters=%i\n", iters);
}

/* ------------------------------------------------------------ vcycle -- */
double vcycle(int giter, int save_tre)
{
   const char *var = AMRD_elliptic_vars[0];
   int Lmg = PAMR_get_max_lev(ABI_PAMR_MGH), Lamr = PAMR_get_max_lev(ABI_PAMR_AMRH);
   int gm, L = 0, m, k, gms[MAXSRC], gres, num_tl = 1, tl, v, nv = AMRD_num_elliptic_vars;
   int gmv[PGB_MAX_VARS], gresv[PGB_MAX_VARS];
   double res = 0;
   vattr a;
   (void)giter;
   if (save_tre) stop("vcycle: save_tre is not supported on the device", "");
   if (Lmg < 1) stop("vcycle: no MG hierarchy (PAMR_build_mgh first)", "");
   if (nv < 1 || nv > PGB_MAX_VARS) stop("vcycle: 1 to 4 elliptic variables", "");
   gm = gfn(var, ABI_PAMR_MGH, 0);
   if (var_attr(var, &a)) num_tl = a.num_tl;
   /* which AMR levels the MG hierarchy replicates: an MG grid of an AMR
    * level holds the AMR grid's own storage (amr_to_mgh aliases it) */
   for (m = Lmg; m >= 1; m--) {
      pgrid g;
      double *p;
      int l, found = 0;
      if (!PAMR_init_s_iter(m, ABI_PAMR_MGH, 0) || !attribs(&g)) break;
      p = g.gfs[gm - 1];
      for (l = Lamr; l >= 1 && !found; l--)
         for (tl = 1; tl <= num_tl && !found; tl++) {
            int ga = gfn(var, ABI_PAMR_AMRH, tl), valid = PAMR_init_s_iter(l, ABI_PAMR_AMRH, 0);
            while (valid && !found) {
               pgrid h;
               attribs(&h);
               if (h.gfs[ga - 1] == p) found = l;
               valid = PAMR_next_g();
            }
         }
      if (!found) break;
      L = found;
   }
   if (!L) stop("vcycle: the MG hierarchy holds no AMR level", "");
   ensure_solver(L, Lamr);
   if (pgb_num_levels(G.s) != Lmg) stop("vcycle: the MG hierarchy differs from the device hierarchy", "");
   for (k = 0; k < G.nsrc; k++) gms[k] = gfn(G.src_names[k], ABI_PAMR_MGH, 0);
   if (G.nvar != nv) stop("vcycle: the device hierarchy carries another number of elliptic variables", "");
   for (v = 0; v < nv; v++) {   /* every elliptic variable and its f_res on the MG hierarchy */
      char rn[512];
      gmv[v] = gfn(AMRD_elliptic_vars[v], ABI_PAMR_MGH, 0);
      snprintf(rn, sizeof(rn), "%s_res", AMRD_elliptic_vars[v]);
      gresv[v] = gfn(rn, ABI_PAMR_MGH, 0);
   }
   gres = gresv[0];
   /* copy in every MG level's u and sources, in PAMR grid-list order */
   for (m = 1; m <= Lmg; m++) {
      int idx = 0, valid = PAMR_init_s_iter(m, ABI_PAMR_MGH, 0);
      while (valid) {
         pgrid g;
         double bb[6], dx[3] = {1, 1, 1};
         int sh[3], d;
         attribs(&g);
         if (idx >= pgb_level_nbox(G.s, m)) stop("vcycle: the MG hierarchy differs from the device hierarchy", "");
         pgb_box_info(G.s, m, idx, sh, bb, 0, 0);
         for (d = 0; d < g.dim; d++) dx[d] = g.x[d][1] - g.x[d][0];
         if (sh[0] != g.shape[0] || sh[1] != g.shape[1] || sh[2] != g.shape[2] || !same_bbox(bb, g.bbox, g.dim, dx))
            stop("vcycle: the MG hierarchy differs from the device hierarchy", "");
         ok_pgb(pgb_box_set(G.s, m, idx, PGB_FIELD_U, g.gfs[gm - 1]), "copying u");
         for (v = 1; v < nv; v++)
            ok_pgb(pgb_box_set(G.s, m, idx, PGB_FIELD_VAR(v) + PGB_FIELD_U, g.gfs[gmv[v] - 1]), "copying a variable");
         for (k = 0; k < G.nsrc; k++)
            ok_pgb(pgb_box_set(G.s, m, idx, PGB_FIELD_SRC + k, g.gfs[gms[k] - 1]), "copying a source");
         idx++;
         valid = PAMR_next_g();
      }
      if (idx != pgb_level_nbox(G.s, m)) stop("vcycle: the MG hierarchy differs from the device hierarchy", "");
   }
   ok_pgb(pgb_prepare_ex(G.s, PGB_PREPARE_KEEP_MG_DATA), "preparing the cycle");
   ok_pgb(pgb_vcycle(G.s, &res), "vcycle");
   /* copy out u everywhere, f_res of the finest level, the boundary cmask */
   for (m = 1; m <= Lmg; m++) {
      int idx = 0, valid = PAMR_init_s_iter(m, ABI_PAMR_MGH, 0);
      while (valid) {
         pgrid g;
         attribs(&g);
         ok_pgb(pgb_box_get(G.s, m, idx, PGB_FIELD_U, g.gfs[gm - 1]), "reading u back");
         if (m == Lmg) ok_pgb(pgb_box_get(G.s, m, idx, PGB_FIELD_RES, g.gfs[gres - 1]), "reading f_res back");
         /* the sources the cycle injected into the pure MG levels, as the
          * reference's vcycle leaves them in PAMR's MG grids */
         for (k = 0; k < G.nsrc && m < Lmg; k++)
            ok_pgb(pgb_box_get(G.s, m, idx, PGB_FIELD_SRC + k, g.gfs[gms[k] - 1]), "reading a source back");
         for (v = 1; v < nv; v++) {
            ok_pgb(pgb_box_get(G.s, m, idx, PGB_FIELD_VAR(v) + PGB_FIELD_U, g.gfs[gmv[v] - 1]), "reading a variable back");
            if (m == Lmg)
               ok_pgb(pgb_box_get(G.s, m, idx, PGB_FIELD_VAR(v) + PGB_FIELD_RES, g.gfs[gresv[v] - 1]),
                      "reading a variable's f_res back");
         }
         if (AMRD_cmask_mg_gfn > 0) put_bdy_mask(m, idx, g.gfs[AMRD_cmask_mg_gfn - 1]);
         idx++;
         valid = PAMR_next_g();
      }
   }
   return res;
}

/* ------------------------------------------- cmask of the AMR hierarchy -- */
/* set_cmask_bdy (amrd/mg.c:432-488) */
void set_cmask_bdy(int L, int hier)
{
   int valid = PAMR_init_s_iter(L, hier, 0);
   const int gc = hier == ABI_PAMR_MGH ? AMRD_cmask_mg_gfn : AMRD_cmask_gfn;
   while (valid) {
      pgrid g;
      int is = 0, js = 0, ks = 0, ie, je = 0, ke = 0, i, j, k;
      long n;
      double *mask, dx[3] = {1, 1, 1};
      attribs(&g);
      mask = g.gfs[gc - 1];
      n = (long)g.shape[0] * g.shape[1] * g.shape[2];
      for (i = 0; i < g.dim; i++) dx[i] = g.x[i][1] - g.x[i][0];
      for (i = 0; i < n; i++) mask[i] = ABI_AMRD_CMASK_OFF;
      ie = g.shape[0] - 1;
      if ((g.bbox[0] - AMRD_base_bbox[0]) > dx[0] / 2 || AMRD_periodic[0]) is++;
      if ((AMRD_base_bbox[1] - g.bbox[1]) > dx[0] / 2 || AMRD_periodic[0]) ie--;
      if (g.dim > 1) {
         je = g.shape[1] - 1;
         if ((g.bbox[2] - AMRD_base_bbox[2]) > dx[1] / 2 || AMRD_periodic[1]) js++;
         if ((AMRD_base_bbox[3] - g.bbox[3]) > dx[1] / 2 || AMRD_periodic[1]) je--;
         if (g.dim > 2) {
            ke = g.shape[2] - 1;
            if ((g.bbox[4] - AMRD_base_bbox[4]) > dx[2] / 2 || AMRD_periodic[2]) ks++;
            if ((AMRD_base_bbox[5] - g.bbox[5]) > dx[2] / 2 || AMRD_periodic[2]) ke--;
         }
      }
      if (is >= 0 && js >= 0 && ks >= 0 && is <= ie && js <= je && ks <= ke && ie < g.shape[0] &&
          je < g.shape[1] && ke < g.shape[2])
         for (i = is; i <= ie; i++)
            for (j = js; j <= je; j++)
               for (k = ks; k <= ke; k++)
                  mask[i + (long)j * g.shape[0] + (long)k * g.shape[0] * g.shape[1]] = ABI_AMRD_CMASK_ON;
      valid = PAMR_next_g();
   }
}

/* extend_cmask_bdy (amrd/mg.c:496-544): an ON point on a grid face whose
 * neighbour num points inward along the face is OFF turns OFF */
void extend_cmask_bdy(int L, int hier, int num)
{
   const double TMP_OFF = -100;
   int valid = PAMR_init_s_iter(L, hier, 0);
   const int gc = hier == ABI_PAMR_MGH ? AMRD_cmask_mg_gfn : AMRD_cmask_gfn;
   while (valid) {
      pgrid g;
      int nx, ny, nz, i, j, k;
      long n;
      double *mask;
      attribs(&g);
      mask = g.gfs[gc - 1];
      nx = g.shape[0];
      ny = g.shape[1];
      nz = g.shape[2];
      n = (long)nx * ny * nz;
#define MI(a, b, c) mask[(a) + (long)(b) * nx + (long)(c) * nx * ny]
      for (i = 0; i < nx; i++) {
         const int ip = i + num < nx - 1 ? i + num : nx - 1, im = i - num > 0 ? i - num : 0;
         for (j = 0; j < ny; j++) {
            const int jp = j + num < ny - 1 ? j + num : ny - 1, jm = j - num > 0 ? j - num : 0;
            for (k = 0; k < nz; k++) {
               const int kp = k + num < nz - 1 ? k + num : nz - 1, km = k - num > 0 ? k - num : 0;
               if (MI(i, j, k) != ABI_AMRD_CMASK_ON) continue;
               if (((j == 0 || j == ny - 1 || k == 0 || k == nz - 1) &&
                    (MI(ip, j, k) == ABI_AMRD_CMASK_OFF || MI(im, j, k) == ABI_AMRD_CMASK_OFF)) ||
                   ((i == 0 || i == nx - 1 || k == 0 || k == nz - 1) &&
                    (MI(i, jp, k) == ABI_AMRD_CMASK_OFF || MI(i, jm, k) == ABI_AMRD_CMASK_OFF)) ||
                   ((i == 0 || i == nx - 1 || j == 0 || j == ny - 1) &&
                    (MI(i, j, kp) == ABI_AMRD_CMASK_OFF || MI(i, j, km) == ABI_AMRD_CMASK_OFF)))
                  MI(i, j, k) = TMP_OFF;
            }
         }
      }
#undef MI
      for (i = 0; i < n; i++)
         if (mask[i] == TMP_OFF) mask[i] = ABI_AMRD_CMASK_OFF;
      valid = PAMR_next_g();
   }
}
