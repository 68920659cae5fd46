/*
 * An nbs-style AMRD application for the drop-in test of libamrd_mg_gb300.
 *
 * Its elliptic equation is the Newtonian boson star's potential,
 * V_xx + V_yy + V_zz - (phi_r^2 + phi_i^2) = 0 (examples/nbs/num.f:85-246),
 * with V = "u" and phi_r, phi_i = "rho", "rho1"; or, in coupled cases, two
 * elliptic variables u and w solved together (the coupled pair of
 * oracle/mg_ops.h, sources "rho", "rho1"), whose hooks handle both. Like examples/nbs/nbs.c it
 * installs host hooks for relax / residual / L_op (here the checker's C
 * restatement of num.f, oracle/mg_ops.c), reads and writes its grids only
 * through the PAMR API, and calls the multigrid module through the
 * reference's entry points:
 *   mode 0  solve_elliptics(L, 1, 0)                       (amrd/mg.c:20)
 *   mode 1  PAMR_build_mgh(Lf, Lf, 1); `arg` times: change the sources of
 *           the finest level, vcycle(k, 0); PAMR_destroy_mgh()
 *           (the evolution iteration's pattern, amrd/evolve.c:454-493)
 * The same source builds two ways: against the reference's own PAMR/AMRD
 * with amrd/mg.c (oracle, where the reference tree exists), and against
 * libamrd_mg_gb300 with -DDEVICE_MG, where the only added line registers
 * the operator for the device. Output: cycle count, residuals, the hook
 * log, and u and cmask of every AMR grid.
 *
 * usage: nbs_app <case.bin> <param file> <out.bin>
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "amrd_abi.h"
#include "mg_ops.h"
#ifdef DEVICE_MG
#include "amrd_mg_gb300.h"
#else
/* amrd/mg.h:32-37 */
void solve_elliptics(int L, int tl, int save_tre);
double vcycle(int giter, int save_tre);
#endif

int PAMR_get_g_level(int *L);
int PAMR_build_mgh(int min_lev, int max_lev, int tl);
int PAMR_destroy_mgh(void);
extern double (*app_MG_residual)(void);
extern double (*app_MG_relax)(void);
extern void (*app_L_op)(void);
extern void (*app_AMRH_var_clear)(void);

/* the environment: the reference's init_context + PAMR_compose_hierarchy
 * (tests/dropin/env_ref.c) or the port's (oracle/port/pamr_env.c) */
int env_init(const char *case_path, const char *param_path);

/* ----------------------------------------------------------------- hooks -- */
typedef struct {
   int dim, shape[3], L;
   double bbox[6], *x[3], *gfs[4096];
} cur;

static void load(cur *g)
{
   int rank, gw[6], ngfs, d;
   double t;
   g->shape[0] = g->shape[1] = g->shape[2] = 1;
   memset(g->bbox, 0, sizeof(g->bbox));
   PAMR_get_g_attribs(&rank, &g->dim, g->shape, g->bbox, gw, &t, &ngfs, g->x, g->gfs);
   PAMR_get_g_level(&g->L);
   for (d = g->dim; d < 3; d++) g->shape[d] = 1;
}

static void ogrid(const cur *g, oracle_grid *o)
{
   int d;
   o->dim = g->dim;
   for (d = 0; d < 3; d++) {
      o->shape[d] = g->shape[d];
      o->dx[d] = d < g->dim ? g->x[d][1] - g->x[d][0] : 1.0;
   }
}

#define MGF(name) (g.gfs[PAMR_get_gfn(name, ABI_PAMR_MGH, 0) - 1])

typedef struct {
   int kind, L;
   double norm;
} hrec;
static hrec *hlog;
static int nh, caph;

static void hlog_add(int kind, int L, double norm)
{
   if (nh == caph) {
      caph = caph ? 2 * caph : 1024;
      hlog = (hrec *)realloc(hlog, sizeof(hrec) * (size_t)caph);
   }
   hlog[nh].kind = kind;
   hlog[nh].L = L;
   hlog[nh].norm = norm;
   nh++;
}

static int coupled;   /* two elliptic variables (u, w) */

static double nbs_MG_relax(void)
{
   cur g;
   oracle_grid o;
   const double *src[2];
   double n;
   load(&g);
   ogrid(&g, &o);
   src[0] = MGF("rho");
   src[1] = MGF("rho1");
   if (coupled) {
      double *v[2] = {MGF("u"), MGF("w")};
      const double *r[2] = {MGF("u_rhs"), MGF("w_rhs")};
      n = oracle_relax_n(ORACLE_COUPLED, &o, v, r, src, MGF("cmask"));
   } else
      n = oracle_relax(ORACLE_NBS, &o, MGF("u"), MGF("u_rhs"), src, MGF("cmask"));
   hlog_add(0, g.L, n);
   return n;
}

static double nbs_MG_residual(void)
{
   cur g;
   oracle_grid o;
   const double *src[2];
   double n;
   load(&g);
   ogrid(&g, &o);
   src[0] = MGF("rho");
   src[1] = MGF("rho1");
   if (coupled) {
      double *rs[2] = {MGF("u_res"), MGF("w_res")};
      const double *r[2] = {MGF("u_rhs"), MGF("w_rhs")}, *v[2] = {MGF("u"), MGF("w")};
      n = oracle_residual_n(ORACLE_COUPLED, &o, rs, r, v, src, MGF("cmask"));
   } else
      n = oracle_residual(ORACLE_NBS, &o, MGF("u_res"), MGF("u_rhs"), MGF("u"), src, MGF("cmask"));
   hlog_add(1, g.L, n);
   return n;
}

static void nbs_L_op(void)
{
   cur g;
   oracle_grid o;
   const double *src[2];
   load(&g);
   ogrid(&g, &o);
   src[0] = MGF("rho");
   src[1] = MGF("rho1");
   if (coupled) {
      double *l[2] = {MGF("u_lop"), MGF("w_lop")};
      const double *v[2] = {MGF("u"), MGF("w")};
      oracle_lop_n(ORACLE_COUPLED, &o, l, v, src, MGF("cmask"));
   } else
      oracle_lop(ORACLE_NBS, &o, MGF("u_lop"), MGF("u"), src, MGF("cmask"));
}

static void nbs_var_clear(void) {}

/* ------------------------------------------------------------------ main -- */
static void scale_finest_sources(double f)
{
   int Lf = PAMR_get_max_lev(ABI_PAMR_AMRH), valid = PAMR_init_s_iter(Lf, ABI_PAMR_AMRH, 0);
   const int g0 = PAMR_get_gfn("rho", ABI_PAMR_AMRH, 1), g1 = PAMR_get_gfn("rho1", ABI_PAMR_AMRH, 1);
   while (valid) {
      cur g;
      long n, i;
      load(&g);
      n = (long)g.shape[0] * g.shape[1] * g.shape[2];
      for (i = 0; i < n; i++) {
         g.gfs[g0 - 1][i] *= f;
         g.gfs[g1 - 1][i] *= 2.0 - f;
      }
      valid = PAMR_next_g();
   }
}

int main(int argc, char **argv)
{
   FILE *fo;
   int mode, arg, L, k, l, iters = 0, nres = 0;
   double res[256];
   if (argc < 4) {
      fprintf(stderr, "usage: %s case.bin param.txt out.bin\n", argv[0]);
      return 2;
   }
   app_MG_relax = nbs_MG_relax;
   app_MG_residual = nbs_MG_residual;
   app_L_op = nbs_L_op;
   app_AMRH_var_clear = nbs_var_clear;
   {
      FILE *f = fopen(argv[1], "rb");
      int h[8];
      if (!f || fread(h, 4, 8, f) != 8) return 2;
      fclose(f);
      mode = h[2];
      arg = h[3];
      L = h[4];
      coupled = h[5];
   }
   if (env_init(argv[1], argv[2])) {
      fprintf(stderr, "nbs_app: environment set-up failed\n");
      return 3;
   }
#ifdef DEVICE_MG
   {
      /* the one line an application adds: its operator, for the device */
      char *src[2] = {"rho", "rho1"};
      if (coupled) {   /* one operator per elliptic variable: u, then w */
         if (!amrd_set_device_MG_operator(2, src, "lap - s0*(u - u1) - s1", "j0 - s0")) return 4;
         if (!amrd_set_device_MG_var_operator(1, "lap - s0*(u - u0)", "j0 - s0")) return 4;
      } else if (!amrd_set_device_MG_operator(2, src, "lap - (s0*s0 + s1*s1)", "j0"))
         return 4;
      if (getenv("NBS_APP_MIXED") && !amrd_set_device_MG_precision(1)) return 4;
   }
#endif
   if (mode == 0) {
      solve_elliptics(L, 1, 0);
      iters = AMRD_curr_MG_iter;
#ifdef DEVICE_MG
      nres = amrd_device_MG_residuals(res, 256);
      if (nres > 256) nres = 256;
#endif
   } else {
      int Lf = PAMR_get_max_lev(ABI_PAMR_AMRH);
      if (!PAMR_build_mgh(Lf, Lf, 1)) return 5;
      for (k = 0; k < arg && k < 256; k++) {
         if (k) scale_finest_sources(1.0 + 0.01 * k);
         res[nres++] = vcycle(k, 0);
      }
      PAMR_destroy_mgh();
      iters = nres;
   }
   fo = fopen(argv[3], "wb");
   if (!fo) return 6;
   fwrite(&iters, 4, 1, fo);
   fwrite(&nres, 4, 1, fo);
   fwrite(res, 8, (size_t)nres, fo);
   fwrite(&nh, 4, 1, fo);
   for (k = 0; k < nh; k++) {
      fwrite(&hlog[k].kind, 4, 1, fo);
      fwrite(&hlog[k].L, 4, 1, fo);
      fwrite(&hlog[k].norm, 8, 1, fo);
   }
   for (l = 1; l <= PAMR_get_max_lev(ABI_PAMR_AMRH); l++) {
      int valid = PAMR_init_s_iter(l, ABI_PAMR_AMRH, 0);
      const int gu = PAMR_get_gfn("u", ABI_PAMR_AMRH, 1), gc = PAMR_get_gfn("cmask", ABI_PAMR_AMRH, 1);
      const int gw_ = coupled ? PAMR_get_gfn("w", ABI_PAMR_AMRH, 1) : 0;
      while (valid) {
         cur g;
         long n;
         load(&g);
         n = (long)g.shape[0] * g.shape[1] * g.shape[2];
         fwrite(&l, 4, 1, fo);
         fwrite(g.shape, 4, 3, fo);
         fwrite(g.bbox, 8, 6, fo);
         fwrite(g.gfs[gu - 1], 8, (size_t)n, fo);
         fwrite(g.gfs[gc - 1], 8, (size_t)n, fo);
         if (coupled) fwrite(g.gfs[gw_ - 1], 8, (size_t)n, fo);
         valid = PAMR_next_g();
      }
   }
   fclose(fo);
   return 0;
}
