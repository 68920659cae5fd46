/*
 * The part of the PAMR and AMRD C interfaces that libamrd_mg_gb300 calls,
 * declared with the reference's signatures (include/pamr.h:14-218,
 * include/amrd.h; `real` is double, include/internal_opts.h:9) so that the
 * library links against an application's libpamr / libamrd unchanged.
 * These are declarations of an existing binary interface, kept identical
 * on purpose; the definitions come from the application's libraries.
 */
#ifndef AMRD_ABI_H
#define AMRD_ABI_H

#define ABI_PAMR_AMRH 1            /* include/pamr.h: hierarchy identifiers */
#define ABI_PAMR_MGH 2
#define ABI_PAMR_MAX_DIM 3
#define ABI_AMRD_CMASK_ON 1.0      /* include/amrd.h:445-446 */
#define ABI_AMRD_CMASK_OFF 0.0

/* PAMR (src/pamr.c) */
int PAMR_get_max_lev(int hier);
int PAMR_init_s_iter(int l, int hier, int all);
int PAMR_next_g(void);
int PAMR_push_iter(void);
int PAMR_pop_iter(void);
int PAMR_get_g_attribs(int *rank, int *dim, int *shape, double *bbox, int *ghost_width, double *t, int *ngfs,
                       double **x, double **gfs);
int PAMR_get_gfn(char *name, int hier, int tl);
int PAMR_get_sgh(double *bbox, int *num, int L);
void PAMR_get_global_bbox(double *bbox);
void PAMR_get_dxdt(int lev, double *dx, double *dt);
int PAMR_get_var_attribs(char *name, int *in_amrh, int *in_mgh, int *num_tl, int *amr_inject, int *amr_interp,
                         int *amr_bdy_interp, int *amr_sync, int *mg_inject, int *mg_interp, int *mg_sync,
                         int *mg_noinj_to_amr, int *regrid_transfer, int *phys_bdy_type);
void PAMR_get_MG_coarse_width(int *min_width);
void PAMR_get_interp_buffer(int *interp_buffer);
void PAMR_get_periodic_bdy(int *periodic);

/* AMRD (amrd/globals.c, amrd/util.c) */
extern int AMRD_num_elliptic_vars;
extern int AMRD_num_elliptic_vars_t0;
extern char *AMRD_elliptic_vars[];
extern int AMRD_MG_max_iter, AMRD_MG_min_iter, AMRD_MG_max_citer;
extern double AMRD_MG_tol, AMRD_MG_crtol, AMRD_MG_w0_r, AMRD_MG_w0_i;
extern int AMRD_MG_pre_swp, AMRD_MG_pst_swp;
extern int AMRD_MG_trace;
extern int AMRD_is_t0;
extern int AMRD_curr_MG_iter;
extern int AMRD_num_MG_cnst_data_vars;
extern int AMRD_cmask_gfn, AMRD_cmask_mg_gfn;
extern double AMRD_base_bbox[];
extern int AMRD_periodic[];
extern int my_rank;
extern void (*app_elliptic_vars_t0_init)(void);
void AMRD_stop(char *err1, char *err2);

#endif
