/*
 * A PAMR / AMRD environment for an application, over the oracle port's
 * hierarchy (mg_port.c): the subset of the PAMR API (include/pamr.h) and
 * of AMRD's globals (include/amrd.h) that libamrd_mg_gb300 and the test
 * application use, so that the drop-in multigrid library can be linked and
 * run where the reference itself is not built (the GPU machine).
 *
 * TEST INFRASTRUCTURE (oracle only): used by tests/dropin/. PAMR_build_mgh
 * here is the port's build_mgh (src/gh.c:1222-1365 restated, pinned against
 * the compiled reference by tests/test_oracle_port.py), so MG hierarchies
 * and their build-time injections are the reference's.
 *
 * Variables: the elliptic variable "u", sources "rho" and "rho1" (as
 * oracle/refrun.py names them), the MG work variables u_res, u_lop, u_rhs
 * and "cmask", one time level. gfn numbering of this environment:
 *   u 1 (AMR) / 2 (MG), rho 3 / 4, rho1 5 / 6, u_res 7, u_lop 8, u_rhs 9,
 *   cmask 10 / 11.
 * A coupled case adds a second elliptic variable "w" (gfn 12 AMR / 13 MG)
 * and its MG residual w_res (14), carried by the port's grids and MG
 * hierarchy like u and u_res (port_carry_second_var), so that both
 * solve_elliptics and vcycle run on such a case.
 */
#include "mg_port.c"
#include "../../tests/dropin/dropin_case.h"

/* ------------------------------------------------------ AMRD globals -- */
int AMRD_num_elliptic_vars = 1, AMRD_num_elliptic_vars_t0 = 0;
char *AMRD_elliptic_vars[4] = {"u", 0, 0, 0};
int AMRD_MG_max_iter, AMRD_MG_min_iter, AMRD_MG_max_citer;
double AMRD_MG_tol, AMRD_MG_crtol, AMRD_MG_w0_r, AMRD_MG_w0_i;
int AMRD_MG_pre_swp, AMRD_MG_pst_swp;
int AMRD_MG_trace = 0, AMRD_is_t0 = 0, AMRD_curr_MG_iter = 0, AMRD_num_MG_cnst_data_vars = 0;
int AMRD_cmask_gfn = 10, AMRD_cmask_mg_gfn = 11;
double AMRD_base_bbox[6];
int AMRD_periodic[3] = {0, 0, 0};
int my_rank = 0;
void (*app_elliptic_vars_t0_init)(void) = 0;
double (*app_MG_residual)(void) = 0;
double (*app_MG_relax)(void) = 0;
void (*app_L_op)(void) = 0;
void (*app_AMRH_var_clear)(void) = 0;

void AMRD_stop(char *err1, char *err2)
{
   printf("%s%s\n", err1 ? err1 : "", err2 ? err2 : "");
   fflush(stdout);
   exit(3);
}

/* ---------------------------------------------------------- the case -- */
static port_case E_case;
static int *E_lev;
static double *E_bbox;
static double **E_u, **E_src, **E_src1;
static const double *E_srcx[1][4096];
/* a coupled case: a second elliptic variable */
static int E_nw;

int env_init(const char *case_path, const char *param_path)
{
   dropin_case dc;
   int i, d;
   (void)param_path;
   if (dropin_read_case(case_path, &dc)) return 2;
   memset(&E_case, 0, sizeof(E_case));
   E_case.dim = dc.dim;
   E_case.pde = ORACLE_NBS;
   E_case.ngrids = dc.ngrids;
   for (d = 0; d < 3; d++) E_case.base_shape[d] = dc.base_shape[d];
   for (d = 0; d < 6; d++) E_case.base_bbox[d] = dc.base_bbox[d];
   E_lev = dc.lev;
   E_bbox = dc.bbox;
   E_u = dc.u;
   E_src = dc.src0;
   E_src1 = dc.src1;
   for (i = 0; i < dc.ngrids && i < 4096; i++) E_srcx[0][i] = E_src1[i];
   E_case.lev = E_lev;
   E_case.bbox = E_bbox;
   E_case.u = E_u;
   E_case.src = (const double *const *)E_src;
   E_case.srcx[0] = E_srcx[0];
   E_case.pre_swp = dc.ip[0];
   E_case.pst_swp = dc.ip[1];
   E_case.max_iter = dc.ip[2];
   E_case.min_iter = dc.ip[3];
   E_case.max_citer = dc.ip[4];
   E_case.min_cwidth = dc.ip[5];
   E_case.restr_u = dc.ip[6];
   E_case.restr_res = dc.ip[7];
   E_case.restr_src = dc.ip[8];
   E_case.restr_srcx[0] = dc.ip[9];
   E_case.tol = dc.fp[0];
   E_case.crtol = dc.fp[1];
   E_case.w0_r = dc.fp[2];
   E_case.w0_i = dc.fp[3];
   E_case.interp_order = 2;
   E_case.interp_buffer = 2;
   E_case.min_level = 1;
   E_nw = dc.coupled != 0;
   port_carry_second_var(E_nw);
   if (port_compose(&E_case, 0)) return 3;
   if (dc.coupled) {   /* w on every AMR grid, from the case */
      int l;
      AMRD_num_elliptic_vars = 2;
      AMRD_elliptic_vars[1] = "w";
      for (l = 1; l <= P.n_amr; l++)
         for (pgrid *g = P.amr[l].grids; g; g = g->next) {
            long n = (long)g->shape[0] * g->shape[1] * g->shape[2];
            for (i = 0; i < dc.ngrids; i++) {
               int same = dc.lev[i] == l, q;
               for (q = 0; q < 2 * dc.dim && same; q++)
                  if (fabs(dc.bbox[6 * i + q] - g->bbox[q]) > 1e-9 * (1 + fabs(g->bbox[q]))) same = 0;
               if (same) break;
            }
            if (i == dc.ngrids || !g->gf[G_W]) return 4;
            memcpy(g->gf[G_W], dc.w[i], sizeof(double) * (size_t)n);
         }
   }
   AMRD_MG_pre_swp = E_case.pre_swp;
   AMRD_MG_pst_swp = E_case.pst_swp;
   AMRD_MG_max_iter = E_case.max_iter;
   AMRD_MG_min_iter = E_case.min_iter;
   AMRD_MG_max_citer = E_case.max_citer;
   AMRD_MG_tol = E_case.tol;
   AMRD_MG_crtol = E_case.crtol;
   AMRD_MG_w0_r = E_case.w0_r;
   AMRD_MG_w0_i = E_case.w0_i;
   for (d = 0; d < 6; d++) AMRD_base_bbox[d] = E_case.base_bbox[d];
   return 0;
}

/* ----------------------------------------------------------- iterators -- */
#define E_MAXSTACK 10
static struct {
   int hier, level;
   pgrid *g;
} E_it, E_stack[E_MAXSTACK];
static int E_sp = 0;

static plev *E_level(int l, int hier)
{
   if (hier == 1 && l >= 1 && l <= P.n_amr) return &P.amr[l];
   if (hier == 2 && l >= 1 && l <= P.n_mg) return &P.mg[l];
   return 0;
}

int PAMR_init_s_iter(int l, int hier, int all)
{
   plev *lv = E_level(l, hier);
   (void)all;
   E_it.hier = hier;
   E_it.level = l;
   E_it.g = lv ? lv->grids : 0;
   return E_it.g != 0;
}

int PAMR_next_g(void)
{
   if (E_it.g) E_it.g = E_it.g->next;
   return E_it.g != 0;
}

int PAMR_push_iter(void)
{
   if (E_sp >= E_MAXSTACK) return 0;
   E_stack[E_sp++] = E_it;
   return 1;
}

int PAMR_pop_iter(void)
{
   if (E_sp <= 0) return 0;
   E_it = E_stack[--E_sp];
   return 1;
}

int PAMR_get_max_lev(int hier) { return hier == 1 ? P.n_amr : P.n_mg; }

int PAMR_get_g_level(int *L)
{
   *L = E_it.level;
   return E_it.g != 0;
}

int PAMR_get_g_attribs(int *rank, int *dim, int *shape, double *bbox, int *ghost_width, double *t, int *ngfs,
                       double **x, double **gfs)
{
   pgrid *g = E_it.g;
   int d;
   if (!g) return 0;
   *rank = 0;
   *dim = P.dim;
   for (d = 0; d < P.dim; d++) {
      shape[d] = g->shape[d];
      bbox[2 * d] = g->bbox[2 * d];
      bbox[2 * d + 1] = g->bbox[2 * d + 1];
      ghost_width[2 * d] = ghost_width[2 * d + 1] = 0;
      x[d] = g->x[d];
   }
   *t = 0;
   *ngfs = 14;
   for (d = 0; d < 14; d++) gfs[d] = 0;
   if (E_it.hier == 1) {
      gfs[11] = g->gf[G_W];
      gfs[0] = g->gf[G_U];
      gfs[2] = g->gf[G_SRC];
      gfs[4] = g->gf[G_SRC1];
      gfs[9] = g->gf[G_CMASK];
   } else {
      gfs[1] = g->gf[G_U];
      gfs[3] = g->gf[G_SRC];
      gfs[5] = g->gf[G_SRC1];
      gfs[6] = g->gf[G_RES];
      gfs[7] = g->gf[G_LOP];
      gfs[8] = g->gf[G_RHS];
      gfs[10] = g->gf[G_CMASK];
      gfs[12] = g->gf[G_W];
      gfs[13] = g->gf[G_WRES];
   }
   return 1;
}

int PAMR_get_gfn(char *name, int hier, int tl)
{
   static const struct {
      const char *n;
      int amr, mg;
   } tab[] = {{"u", 1, 2}, {"rho", 3, 4}, {"rho1", 5, 6}, {"u_res", 0, 7}, {"u_lop", 0, 8},
              {"u_rhs", 0, 9}, {"cmask", 10, 11}, {"w", 12, 13}, {"w_res", 0, 14}};
   int i;
   for (i = 0; i < (int)(sizeof(tab) / sizeof(tab[0])); i++)
      if (!strcmp(name, tab[i].n)) {
         int g = hier == 1 ? (tl == 1 ? tab[i].amr : 0) : tab[i].mg;
         return g ? g : -1;
      }
   return -1;
}

int PAMR_get_sgh(double *bbox, int *num, int L)
{
   int n, i;
   if (L < 1 || L > P.n_amr) return 0;
   n = P.sgh_num[L] < *num ? P.sgh_num[L] : *num;
   *num = n;
   for (i = 0; i < 2 * P.dim * n; i++) bbox[i] = P.sgh_bbox[L][i];
   return 1;
}

void PAMR_get_global_bbox(double *bbox)
{
   int i;
   for (i = 0; i < 2 * P.dim; i++) bbox[i] = P.bbox[i];
}

void PAMR_get_dxdt(int lev, double *dx, double *dt)
{
   int d;
   for (d = 0; d < P.dim; d++) dx[d] = P.amr_dx[lev][d];
   *dt = 0;
}

int PAMR_get_var_attribs(char *name, int *in_amrh, int *in_mgh, int *num_tl, int *amr_inject, int *amr_interp,
                         int *amr_bdy_interp, int *amr_sync, int *mg_inject, int *mg_interp, int *mg_sync,
                         int *mg_noinj_to_amr, int *regrid_transfer, int *phys_bdy_type)
{
   (void)phys_bdy_type;
   *amr_inject = *amr_interp = *amr_bdy_interp = *amr_sync = *regrid_transfer = 0;
   *num_tl = 1;
   *mg_interp = *mg_sync = *mg_noinj_to_amr = 0;
   *in_amrh = *in_mgh = 1;
   if (!strcmp(name, "u") || (E_nw && !strcmp(name, "w"))) {
      *mg_inject = P.c->restr_u;
      *mg_sync = 1;
   } else if (!strcmp(name, "u_res") || (E_nw && !strcmp(name, "w_res"))) {
      *in_amrh = 0;
      *mg_inject = P.c->restr_res;
      *mg_interp = P.c->interp_order;
   } else if (!strcmp(name, "rho")) {
      *mg_inject = P.c->restr_src;
      *mg_noinj_to_amr = 1;
   } else if (!strcmp(name, "rho1")) {
      *mg_inject = P.c->restr_srcx[0];
      *mg_noinj_to_amr = 1;
   } else if (!strcmp(name, "u_lop") || !strcmp(name, "u_rhs") ||
              (E_nw && (!strcmp(name, "w_lop") || !strcmp(name, "w_rhs")))) {
      *in_amrh = 0;
      *mg_inject = 0;
   } else if (!strcmp(name, "cmask")) {
      *mg_inject = 0;
      *mg_noinj_to_amr = 1;
   } else
      return 0;
   return 1;
}

void PAMR_get_MG_coarse_width(int *min_width)
{
   int d;
   for (d = 0; d < P.dim; d++) min_width[d] = P.c->min_cwidth;
}

void PAMR_get_interp_buffer(int *interp_buffer) { *interp_buffer = P.c->interp_buffer; }

void PAMR_get_periodic_bdy(int *periodic)
{
   int d;
   for (d = 0; d < P.dim; d++) periodic[d] = 0;
}

int PAMR_build_mgh(int min_lev, int max_lev, int tl)
{
   (void)tl;
   if (min_lev < 1 || max_lev != P.n_amr || min_lev > max_lev) return 0;
   P.min_level = min_lev;
   build_mgh();
   return 1;
}

int PAMR_destroy_mgh(void)
{
   destroy_mgh();
   return 1;
}
