/*
 * Driver that runs the REFERENCE's own multigrid solve (amrd/mg.c
 * solve_elliptics over PAMR's MG hierarchy) on a seeded case, and records
 * what a GPU implementation must reproduce.
 *
 * TEST INFRASTRUCTURE (oracle only). Built by oracle/build_ref.sh from the
 * reference's C sources in place (src/pamr.c, src/gh.c, src/transfer.c,
 * src/misc.c, src/io.c, amrd/*.c), the single-rank shims in oracle/shim and
 * the C restatement of the Fortran kernels (oracle/m_util_r8.c). Output goes
 * to oracle/_ref/ only.
 *
 * usage: ref_mg <param file> <case.bin> <out.bin> [log_ops [interp:lc:width]]
 *
 * The parameter file is an AMRD run-time file read by the reference's
 * init_context() (amrd/io.c:36). case.bin carries the AMR hierarchy and the
 * initial u and source on every AMR grid. The driver then
 *   1. composes the hierarchy with PAMR_compose_hierarchy (src/pamr.c:259),
 *   2. fills u and the source on time level 1,
 *   3. calls solve_elliptics(1,1,0) (amrd/mg.c:20), or with interp:lc:width
 *      one PAMR_interp (width 0) or PAMR_AMR_bdy_interp (width > 0) of u
 *      from AMR level lc to lc+1 instead, or with regrid:min_lev:new.bin a
 *      second PAMR_compose_hierarchy (src/pamr.c:257) over levels min_lev..
 *      of the grids of new.bin, whose init_new_cgh (src/gh.c:934) moves u
 *      and the sources (regrid_transfer order from the parameter file) onto
 *      the new grids, which are then written out (tag 9-11),
 * while the application hooks (pattern of examples/nbs/nbs.c:301-351) log
 * every relax/residual norm, the MG hierarchy, the cmask arrays, and (with
 * log_ops) every m_util_r8 call with its index arguments.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "pamr.h"
#include "amrd.h"
#include "mg.h"
#include "mpi.h"
#include "mg_ops.h"
#include "m_util_r8_c.h"

/* amrd/io.c:36 (the reference declares it in amrd/io.h, shadowed here by src/io.h) */
void init_context(char *pfile);

/* ------------------------------------------------------------ case data -- */
typedef struct {
   int lev;
   double bbox[6];
   int shape[3];
   long n;
   double *u, *uv[2], *src[4];   /* u = uv[0]; uv[1]: the second elliptic variable */
} case_grid;

static int c_dim, c_pde, c_ngrids, c_nsrc, c_min_level, c_nvar;
/* names of the elliptic variables in the parameter file (oracle/refrun.py) */
static const char *const VAR_NAMES[2] = {"u", "w"};
/* names of the source variables in the parameter file (oracle/refrun.py) */
static const char *const SRC_NAMES[4] = {"rho", "rho1", "rho2", "rho3"};
static case_grid *c_grids;

/* --------------------------------------------------------------- output -- */
static FILE *fout;
static void rec(int tag, const void *p, long nbytes)
{
   fwrite(&tag, 4, 1, fout);
   fwrite(&nbytes, 8, 1, fout);
   if (nbytes) fwrite(p, 1, (size_t)nbytes, fout);
}

/* ------------------------------------------------------------ hook state -- */
static int gfn_u, gfn_res, gfn_lop, gfn_rhs, gfn_cmask, gfn_src, gfn_srck[4];
/* MG gfns of every elliptic variable (index 0 = gfn_u .. gfn_rhs) */
static int gfn_uv[2], gfn_resv[2], gfn_lopv[2], gfn_rhsv[2];

/* MG hierarchy map, captured at the first hook call */
#define MAXG 4096
typedef struct {
   int L, idx, shape[3], coarsest;
   double bbox[6];
   double *gfs[PAMR_MAX_GFNS];
   int ngfs;
   int have_child_mask, have_bdy_mask;
} mg_grid_rec;
static mg_grid_rec mgmap[MAXG];
static int n_mgmap = 0, mgh_levels = 0;

static int same_bbox(const double *a, const double *b, int dim)
{
   int i;
   for (i = 0; i < 2 * dim; i++)
      if (fabs(a[i] - b[i]) > 1e-9 * (1 + fabs(a[i]))) return 0;
   return 1;
}

static void capture_mgh(void)
{
   int L, valid, idx;
   if (n_mgmap) return;
   mgh_levels = PAMR_get_max_lev(PAMR_MGH);
   PAMR_push_iter();
   for (L = 1; L <= mgh_levels; L++) {
      idx = 0;
      valid = PAMR_init_s_iter(L, PAMR_MGH, 1);
      while (valid) {
         mg_grid_rec *r = &mgmap[n_mgmap++];
         int rank, dim, gw[6], ngfs;
         double t, *x[3];
         r->shape[0] = r->shape[1] = r->shape[2] = 1;
         PAMR_get_g_attribs(&rank, &dim, r->shape, r->bbox, gw, &t, &ngfs, x, r->gfs);
         PAMR_get_g_coarsest(&r->coarsest);
         r->ngfs = ngfs;
         r->L = L;
         r->idx = idx++;
         r->have_child_mask = r->have_bdy_mask = 0;
         valid = PAMR_next_g();
      }
   }
   PAMR_pop_iter();
}

typedef struct {
   int dim, shape[3], L, idx;
   double bbox[6], dx[3];
   double *gfs[PAMR_MAX_GFNS];
   mg_grid_rec *rec;
} cur_grid;

static void ldptr(cur_grid *g)
{
   int rank, gw[6], ngfs, i;
   double t, *x[3];
   g->shape[0] = g->shape[1] = g->shape[2] = 1;
   if (!PAMR_get_g_attribs(&rank, &g->dim, g->shape, g->bbox, gw, &t, &ngfs, x, g->gfs)) {
      fprintf(stderr, "ref_mg: PAMR_get_g_attribs failed\n");
      exit(2);
   }
   PAMR_get_g_level(&g->L);
   for (i = 0; i < 3; i++) g->dx[i] = 1;
   for (i = 0; i < g->dim; i++) g->dx[i] = x[i][1] - x[i][0];
   capture_mgh();
   g->rec = 0;
   g->idx = -1;
   for (i = 0; i < n_mgmap; i++)
      if (mgmap[i].L == g->L && same_bbox(mgmap[i].bbox, g->bbox, g->dim)) {
         g->rec = &mgmap[i];
         g->idx = mgmap[i].idx;
      }
}

static void to_ogrid(const cur_grid *g, oracle_grid *o)
{
   int i;
   o->dim = g->dim;
   for (i = 0; i < 3; i++) {
      o->shape[i] = g->shape[i];
      o->dx[i] = g->dx[i];
   }
}

/* hook log: kind (0 relax, 1 residual, 2 lop), level, grid index, norm */
typedef struct { int kind, L, idx, pad; double norm; } hook_rec;
static hook_rec *hlog;
static int n_hlog = 0, cap_hlog = 0;
static void hook_log(int kind, const cur_grid *g, double norm)
{
   if (n_hlog == cap_hlog) {
      cap_hlog = cap_hlog ? 2 * cap_hlog : 4096;
      hlog = (hook_rec *)realloc(hlog, sizeof(hook_rec) * (size_t)cap_hlog);
   }
   hlog[n_hlog].kind = kind;
   hlog[n_hlog].L = g->L;
   hlog[n_hlog].idx = g->idx;
   hlog[n_hlog].pad = 0;
   hlog[n_hlog].norm = norm;
   n_hlog++;
}

/* masks: stored once per (grid, kind) */
typedef struct { int kind, L, idx, n; double *m; } mask_rec;
static mask_rec masks[2 * MAXG];
static int n_masks = 0;
static void keep_mask(int kind, cur_grid *g)
{
   long n = (long)g->shape[0] * g->shape[1] * g->shape[2];
   mask_rec *m;
   if (!g->rec) return;
   if (kind == 0 && g->rec->have_bdy_mask) return;
   if (kind == 1 && g->rec->have_child_mask) return;
   if (kind == 0) g->rec->have_bdy_mask = 1; else g->rec->have_child_mask = 1;
   m = &masks[n_masks++];
   m->kind = kind;
   m->L = g->L;
   m->idx = g->idx;
   m->n = (int)n;
   m->m = (double *)malloc(sizeof(double) * (size_t)n);
   memcpy(m->m, g->gfs[gfn_cmask - 1], sizeof(double) * (size_t)n);
}

/* the MG instances of the sources on the hook's grid */
static const double *const *grid_src(cur_grid *g)
{
   static double *sv[4];
   int k;
   for (k = 0; k < c_nsrc; k++) sv[k] = g->gfs[gfn_srck[k] - 1];
   return (const double *const *)sv;
}

static double h_relax(void)
{
   cur_grid g;
   oracle_grid o;
   double norm;
   ldptr(&g);
   to_ogrid(&g, &o);
   keep_mask(0, &g);
   if (c_nvar > 1) {
      double *v[2] = {g.gfs[gfn_uv[0] - 1], g.gfs[gfn_uv[1] - 1]};
      const double *r[2] = {g.gfs[gfn_rhsv[0] - 1], g.gfs[gfn_rhsv[1] - 1]};
      norm = oracle_relax_n(c_pde, &o, v, r, grid_src(&g), g.gfs[gfn_cmask - 1]);
   } else
      norm = oracle_relax(c_pde, &o, g.gfs[gfn_u - 1], g.gfs[gfn_rhs - 1], grid_src(&g), g.gfs[gfn_cmask - 1]);
   hook_log(0, &g, norm);
   return norm;
}

static double h_residual(void)
{
   cur_grid g;
   oracle_grid o;
   double norm;
   ldptr(&g);
   to_ogrid(&g, &o);
   if (c_nvar > 1) {
      double *rs[2] = {g.gfs[gfn_resv[0] - 1], g.gfs[gfn_resv[1] - 1]};
      const double *r[2] = {g.gfs[gfn_rhsv[0] - 1], g.gfs[gfn_rhsv[1] - 1]};
      const double *v[2] = {g.gfs[gfn_uv[0] - 1], g.gfs[gfn_uv[1] - 1]};
      norm = oracle_residual_n(c_pde, &o, rs, r, v, grid_src(&g), g.gfs[gfn_cmask - 1]);
   } else
      norm = oracle_residual(c_pde, &o, g.gfs[gfn_res - 1], g.gfs[gfn_rhs - 1], g.gfs[gfn_u - 1],
                             grid_src(&g), g.gfs[gfn_cmask - 1]);
   hook_log(1, &g, norm);
   return norm;
}

static void h_lop(void)
{
   cur_grid g;
   oracle_grid o;
   ldptr(&g);
   to_ogrid(&g, &o);
   keep_mask(1, &g);
   if (c_nvar > 1) {
      double *l[2] = {g.gfs[gfn_lopv[0] - 1], g.gfs[gfn_lopv[1] - 1]};
      const double *v[2] = {g.gfs[gfn_uv[0] - 1], g.gfs[gfn_uv[1] - 1]};
      oracle_lop_n(c_pde, &o, l, v, grid_src(&g), g.gfs[gfn_cmask - 1]);
   } else
      oracle_lop(c_pde, &o, g.gfs[gfn_lop - 1], g.gfs[gfn_u - 1], grid_src(&g), g.gfs[gfn_cmask - 1]);
   hook_log(2, &g, 0);
}

static void h_noop(void) {}

/* ------------------------------------------------------------- case i/o -- */
static void read_case(const char *path)
{
   FILE *f = fopen(path, "rb");
   int i, hdr[4];
   if (!f) { fprintf(stderr, "ref_mg: cannot open %s\n", path); exit(2); }
   if (fread(hdr, 4, 4, f) != 4) exit(2);
   c_dim = hdr[0];
   c_pde = hdr[1];
   c_ngrids = hdr[2];
   c_min_level = hdr[3] > 0 ? hdr[3] : 1;
   c_nsrc = oracle_nsrc(c_pde);
   c_nvar = oracle_nvar(c_pde);
   c_grids = (case_grid *)calloc((size_t)c_ngrids, sizeof(case_grid));
   for (i = 0; i < c_ngrids; i++) {
      case_grid *g = &c_grids[i];
      if (fread(&g->lev, 4, 1, f) != 1) exit(2);
      if (fread(g->shape, 4, 3, f) != 3) exit(2);
      if (fread(g->bbox, 8, 6, f) != 6) exit(2);
      g->n = (long)g->shape[0] * g->shape[1] * g->shape[2];
      {
         int q;
         for (q = 0; q < c_nvar; q++) {   /* every elliptic variable, then the sources */
            g->uv[q] = (double *)malloc(sizeof(double) * (size_t)g->n);
            if (fread(g->uv[q], 8, (size_t)g->n, f) != (size_t)g->n) exit(2);
         }
         g->u = g->uv[0];
      }
      {
         int k;
         for (k = 0; k < c_nsrc; k++) {
            g->src[k] = (double *)malloc(sizeof(double) * (size_t)g->n);
            if (fread(g->src[k], 8, (size_t)g->n, f) != (size_t)g->n) exit(2);
         }
      }
   }
   fclose(f);
}

static case_grid *match_case_grid(int L, const double *bbox, const int *shape)
{
   int i;
   for (i = 0; i < c_ngrids; i++)
      if (c_grids[i].lev == L && same_bbox(c_grids[i].bbox, bbox, c_dim)) {
         if (c_grids[i].shape[0] != shape[0] || c_grids[i].shape[1] != shape[1] ||
             c_grids[i].shape[2] != shape[2]) {
            fprintf(stderr, "ref_mg: shape mismatch on level %i\n", L);
            exit(2);
         }
         return &c_grids[i];
      }
   fprintf(stderr, "ref_mg: no case grid for a level-%i PAMR grid\n", L);
   exit(2);
   return 0;
}

/* fill (dir=0) or read back (dir=1) u and the sources on every AMR grid */
static int g_amr_var[2];   /* AMR gfns (time level 1) of the elliptic variables */
static void amr_data(int dir, int gu, const int *gs)
{
   int L, valid, Lmax = PAMR_get_max_lev(PAMR_AMRH);
   for (L = 1; L <= Lmax; L++) {
      valid = PAMR_init_s_iter(L, PAMR_AMRH, 0);
      while (valid) {
         int rank, dim, gw[6], ngfs, shape[3] = {1, 1, 1};
         double t, *x[3], bbox[6], *gfs[PAMR_MAX_GFNS];
         case_grid *cg;
         PAMR_get_g_attribs(&rank, &dim, shape, bbox, gw, &t, &ngfs, x, gfs);
         cg = match_case_grid(L, bbox, shape);
         if (dir == 0) {
            int k;
            memcpy(gfs[gu - 1], cg->u, sizeof(double) * (size_t)cg->n);
            for (k = 1; k < c_nvar; k++) memcpy(gfs[g_amr_var[k] - 1], cg->uv[k], sizeof(double) * (size_t)cg->n);
            for (k = 0; k < c_nsrc; k++) memcpy(gfs[gs[k] - 1], cg->src[k], sizeof(double) * (size_t)cg->n);
         } else {
            int k;
            memcpy(cg->u, gfs[gu - 1], sizeof(double) * (size_t)cg->n);
            for (k = 1; k < c_nvar; k++) memcpy(cg->uv[k], gfs[g_amr_var[k] - 1], sizeof(double) * (size_t)cg->n);
         }
         valid = PAMR_next_g();
      }
   }
}

/* pointer -> (level, grid index, gfn) for the op log; -1 if a temporary.
 * MG grids on AMR levels alias AMR time-level storage, so the MG-instance
 * gfns are matched first. */
static void resolve(const double *p, int *out)
{
   int i, h, q, np = 6;
   int pref[9];
   pref[0] = gfn_src; pref[1] = gfn_u; pref[2] = gfn_res;
   pref[3] = gfn_lop; pref[4] = gfn_rhs; pref[5] = gfn_cmask;
   for (q = 1; q < c_nsrc; q++) pref[np++] = gfn_srck[q];
   out[0] = out[1] = out[2] = -1;
   for (i = 0; i < n_mgmap; i++)
      for (q = 0; q < np; q++)
         if (mgmap[i].gfs[pref[q] - 1] == p) {
            out[0] = mgmap[i].L;
            out[1] = mgmap[i].idx;
            out[2] = pref[q];
            return;
         }
   for (i = 0; i < n_mgmap; i++)
      for (h = 0; h < mgmap[i].ngfs; h++)
         if (mgmap[i].gfs[h] == p) {
            out[0] = mgmap[i].L;
            out[1] = mgmap[i].idx;
            out[2] = h + 1;
            return;
         }
}

int main(int argc, char **argv)
{
   int i, num, *lev;
   double *bbox;
   int gu_amr, gs_amr[4], k;
   int amr_lc = 0, amr_width = -1, regrid_min = 0;
   char regrid_case[1024] = "";
   if (argc < 4) {
      fprintf(stderr, "usage: %s pfile case.bin out.bin [log_ops [interp:lc:width | regrid:min_lev:new.bin]]\n",
              argv[0]);
      return 2;
   }
   if (argc > 5 && !strncmp(argv[5], "regrid:", 7)) {
      if (sscanf(argv[5], "regrid:%d:%1000s", &regrid_min, regrid_case) != 2 || regrid_min < 1) {
         fprintf(stderr, "ref_mg: bad regrid mode %s\n", argv[5]);
         return 2;
      }
   } else if (argc > 5 && sscanf(argv[5], "interp:%d:%d", &amr_lc, &amr_width) != 2) {
      fprintf(stderr, "ref_mg: bad interpolation mode %s\n", argv[5]);
      return 2;
   }
   read_case(argv[2]);

   MPI_Init(&argc, &argv);
   my_rank = 0;
   app_AMRH_var_clear = h_noop;
   app_MG_relax = h_relax;
   app_MG_residual = h_residual;
   app_L_op = h_lop;

   init_context(argv[1]);

   num = c_ngrids;
   lev = (int *)malloc(sizeof(int) * (size_t)num);
   bbox = (double *)malloc(sizeof(double) * 6 * (size_t)num);
   for (i = 0; i < num; i++) {
      lev[i] = c_grids[i].lev;
      memcpy(&bbox[2 * c_dim * i], c_grids[i].bbox, sizeof(double) * 2 * (size_t)c_dim);
   }
   {
      int nlev = 1;
      for (i = 0; i < num; i++) if (lev[i] > nlev) nlev = lev[i];
      if (!PAMR_compose_hierarchy(1, nlev, num, lev, bbox, 0.0)) {
         fprintf(stderr, "ref_mg: PAMR_compose_hierarchy failed\n");
         return 3;
      }
   }

   gu_amr = PAMR_get_gfn("u", PAMR_AMRH, 1);
   for (k = 0; k < c_nsrc; k++) {
      gs_amr[k] = PAMR_get_gfn((char *)SRC_NAMES[k], PAMR_AMRH, 1);
      gfn_srck[k] = PAMR_get_gfn((char *)SRC_NAMES[k], PAMR_MGH, 0);
      if (gs_amr[k] < 0 || gfn_srck[k] < 0) {
         fprintf(stderr, "ref_mg: source variable %s missing\n", SRC_NAMES[k]);
         return 3;
      }
   }
   gfn_u = PAMR_get_gfn("u", PAMR_MGH, 0);
   gfn_res = PAMR_get_gfn("u_res", PAMR_MGH, 0);
   gfn_lop = PAMR_get_gfn("u_lop", PAMR_MGH, 0);
   gfn_rhs = PAMR_get_gfn("u_rhs", PAMR_MGH, 0);
   gfn_cmask = PAMR_get_gfn("cmask", PAMR_MGH, 0);
   gfn_src = PAMR_get_gfn("rho", PAMR_MGH, 0);
   gfn_uv[0] = gfn_u; gfn_resv[0] = gfn_res; gfn_lopv[0] = gfn_lop; gfn_rhsv[0] = gfn_rhs;
   for (k = 1; k < c_nvar; k++) {
      char nm[32];
      g_amr_var[k] = PAMR_get_gfn((char *)VAR_NAMES[k], PAMR_AMRH, 1);
      gfn_uv[k] = PAMR_get_gfn((char *)VAR_NAMES[k], PAMR_MGH, 0);
      snprintf(nm, sizeof(nm), "%s_res", VAR_NAMES[k]); gfn_resv[k] = PAMR_get_gfn(nm, PAMR_MGH, 0);
      snprintf(nm, sizeof(nm), "%s_lop", VAR_NAMES[k]); gfn_lopv[k] = PAMR_get_gfn(nm, PAMR_MGH, 0);
      snprintf(nm, sizeof(nm), "%s_rhs", VAR_NAMES[k]); gfn_rhsv[k] = PAMR_get_gfn(nm, PAMR_MGH, 0);
      if (g_amr_var[k] < 0 || gfn_uv[k] < 0 || gfn_resv[k] < 0 || gfn_lopv[k] < 0 || gfn_rhsv[k] < 0) {
         fprintf(stderr, "ref_mg: elliptic variable %s missing\n", VAR_NAMES[k]);
         return 3;
      }
   }
   if (gu_amr < 0 || gfn_u < 0 || gfn_res < 0 || gfn_lop < 0 || gfn_rhs < 0 ||
       gfn_cmask < 0 || gfn_src < 0) {
      fprintf(stderr, "ref_mg: missing variable definitions\n");
      return 3;
   }
   amr_data(0, gu_amr, gs_amr);

   mur8_log_enabled = (argc > 4 && atoi(argv[4]));
   if (regrid_min > 0) {
      /* the regrid: the new grids of levels >= regrid_min, composed over the
       * current hierarchy (the levels below stay) */
      int n2 = 0, nl2 = 1, j;
      read_case(regrid_case);   /* the new grids (their data is not used) */
      lev = (int *)realloc(lev, sizeof(int) * (size_t)c_ngrids);
      bbox = (double *)realloc(bbox, sizeof(double) * 6 * (size_t)c_ngrids);
      for (i = 0; i < c_ngrids; i++) {
         if (c_grids[i].lev > nl2) nl2 = c_grids[i].lev;
         if (c_grids[i].lev >= regrid_min) {
            lev[n2] = c_grids[i].lev;
            memcpy(&bbox[2 * c_dim * n2], c_grids[i].bbox, sizeof(double) * 2 * (size_t)c_dim);
            n2++;
         }
      }
      if (!PAMR_compose_hierarchy(regrid_min, nl2, n2, lev, bbox, 0.0)) {
         fprintf(stderr, "ref_mg: regrid PAMR_compose_hierarchy failed\n");
         return 3;
      }
      fout = fopen(argv[3], "wb");
      if (!fout) return 4;
      for (j = 1; j <= PAMR_get_max_lev(PAMR_AMRH); j++) {
         int valid = PAMR_init_s_iter(j, PAMR_AMRH, 0);
         while (valid) {
            int rank, dim, gw[6], ngfs, shape[3] = {1, 1, 1};
            double t, *x[3], gb[6] = {0, 0, 0, 0, 0, 0}, *gfs[PAMR_MAX_GFNS];
            struct { int L, shape[3]; double bbox[6]; } r;
            long n;
            PAMR_get_g_attribs(&rank, &dim, shape, gb, gw, &t, &ngfs, x, gfs);
            n = (long)shape[0] * shape[1] * shape[2];
            r.L = j;
            memcpy(r.shape, shape, sizeof(r.shape));
            memcpy(r.bbox, gb, sizeof(r.bbox));
            rec(9, &r, sizeof(r));
            rec(10, gfs[gu_amr - 1], 8 * n);
            for (k = 0; k < c_nsrc; k++) rec(11, gfs[gs_amr[k] - 1], 8 * n);
            valid = PAMR_next_g();
         }
      }
      fclose(fout);
      return 0;
   }
   if (amr_width >= 0) {
      /* instead of the solve: one AMR-hierarchy interpolation of u (time
       * level 1) from level amr_lc to amr_lc+1, over the whole overlap
       * (PAMR_interp, src/pamr.c:623) or a boundary band of the fine grids
       * (PAMR_AMR_bdy_interp, src/pamr.c:645) */
      int ok = amr_width == 0 ? PAMR_interp(amr_lc, 1, PAMR_AMRH) : PAMR_AMR_bdy_interp(amr_lc, 1, amr_width);
      if (!ok) {
         fprintf(stderr, "ref_mg: AMR interpolation failed\n");
         return 3;
      }
   } else
      solve_elliptics(c_min_level, 1, 0);
   mur8_log_enabled = 0;

   amr_data(1, gu_amr, gs_amr);

   fout = fopen(argv[3], "wb");
   if (!fout) return 4;
   {
      int gf[9] = {gfn_u, gfn_res, gfn_lop, gfn_rhs, gfn_cmask, gfn_src, 0, 0, 0};
      for (k = 1; k < c_nsrc; k++) gf[5 + k] = gfn_srck[k];
      rec(1, &AMRD_curr_MG_iter, 4);
      rec(2, gf, sizeof(gf));
      rec(3, hlog, (long)sizeof(hook_rec) * n_hlog);
   }
   /* MG hierarchy: per grid L, idx, shape[3], coarsest, bbox[6] */
   for (i = 0; i < n_mgmap; i++) {
      struct { int L, idx, shape[3], coarsest; double bbox[6]; } r;
      r.L = mgmap[i].L;
      r.idx = mgmap[i].idx;
      memcpy(r.shape, mgmap[i].shape, sizeof(r.shape));
      r.coarsest = mgmap[i].coarsest;
      memcpy(r.bbox, mgmap[i].bbox, sizeof(r.bbox));
      rec(4, &r, sizeof(r));
   }
   for (i = 0; i < n_masks; i++) {
      int h[4] = {masks[i].kind, masks[i].L, masks[i].idx, masks[i].n};
      rec(5, h, sizeof(h));
      rec(6, masks[i].m, 8L * masks[i].n);
   }
   for (i = 0; i < c_ngrids; i++) rec(7, c_grids[i].u, 8 * c_grids[i].n);
   for (k = 1; k < c_nvar; k++)   /* the other elliptic variables, grid by grid */
      for (i = 0; i < c_ngrids; i++) rec(12, c_grids[i].uv[k], 8 * c_grids[i].n);
   {
      for (i = 0; i < mur8_log_n; i++) {
         int r[4 + 6 + MUR8_NARGS];
         r[0] = mur8_log[i].kind;
         r[1] = r[2] = r[3] = 0;
         resolve(mur8_log[i].u1, &r[4]);
         resolve(mur8_log[i].u2, &r[7]);
         memcpy(&r[10], mur8_log[i].iv, sizeof(int) * MUR8_NARGS);
         rec(8, r, sizeof(r));
      }
   }
   fclose(fout);
   return 0;
}
