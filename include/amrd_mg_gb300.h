/*
 * amrd_mg_gb300.h --- libamrd_mg_gb300: a drop-in replacement of AMRD's
 * multigrid module (amrd/mg.c) that runs the elliptic solve on a GB300
 * through libpamr_gb300.
 *
 * An AMRD application links this library in place of amrd/mg.o and keeps
 * its call sites: AMRD's Berger-Oliger driver (amrd/evolve.c) and the
 * application call the same functions with the same signatures
 * (amrd/mg.h:32-37 and the helpers evolve.c/cls.c use). The library reads
 * the hierarchy and the grid functions through the PAMR API of the
 * application's libpamr (iterators, PAMR_get_g_attribs, PAMR_get_gfn,
 * PAMR_get_sgh; include/pamr.h) and the MG parameters from AMRD's globals
 * (include/amrd.h:264-279), copies them to the device, solves there, and
 * writes the results back into PAMR's host arrays. Nothing is linked from
 * the reference into this library.
 *
 * The one addition an application makes: its elliptic operator for the
 * device, registered once before the first solve (the host hooks
 * app_MG_relax / app_MG_residual / app_L_op stay as they are; the device
 * path does not call them):
 *
 *    char *src[2] = {"phi_r", "phi_i"};
 *    amrd_set_device_MG_operator(2, src, "lap - (s0*s0 + s1*s1)", "j0");
 *
 * (the nbs potential of examples/nbs/num.f:85-246; expression syntax in
 * pamr_gb300.h, pgb_operator_create). Errors are reported the AMRD way:
 * a message and AMRD_stop (amrd/util.c:27-34).
 */
#ifndef AMRD_MG_GB300_H
#define AMRD_MG_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* --- the reference's entry points (same names, arguments and meaning) --- */

/* Solves the elliptic equations on AMR levels L..Lf at time level tl
 * (amrd/mg.c:20-79): V-cycles until the finest residual is <= AMRD_MG_tol
 * (at least AMRD_MG_min_iter, at most AMRD_MG_max_iter); sets
 * AMRD_curr_MG_iter. The elliptic variable on levels L..Lf (time level
 * tl) and the AMR cmask of those levels hold what the reference's solve
 * leaves there. save_tre must be 0 (truncation-error estimates are not
 * computed on the device). */
void solve_elliptics(int L, int tl, int save_tre);

/* One FAS V-cycle on the MG hierarchy the caller built with PAMR_build_mgh
 * (amrd/mg.c:84-201; called once per evolution iteration,
 * amrd/evolve.c:454-487); returns the finest level's residual. The MG
 * hierarchy's elliptic variable on every MG level and f_res on the finest
 * level hold the reference's values afterwards (the other MG work
 * variables are scratch of the device solve and are not copied back). */
double vcycle(int giter, int save_tre);

/* set_cmask_bdy / extend_cmask_bdy of amrd/mg.c:432-544, which AMRD's
 * evolve.c and cls.c call on the AMR hierarchy: cmask ON at interior and
 * physical-boundary points of level L's grids; extend the OFF band by num
 * points from AMR boundaries. Host arrays, as in the reference. */
void set_cmask_bdy(int L, int hier);
void extend_cmask_bdy(int L, int hier, int num);

/* --- additions ------------------------------------------------------ */

/* The device form of the application's MG operator (see above): nsrc
 * source variables by AMRD/PAMR name (read at the solve's time level),
 * L[u] and dL/du as expressions. Returns 1 on success, 0 on failure (PAMR
 * convention) with a message printed. */
int amrd_set_device_MG_operator(int nsrc, char **src_names, char *lop, char *jac);

/* With several elliptic variables (AMRD_num_elliptic_vars > 1): the device
 * operator of variable var (1.., the order of AMRD_elliptic_vars), on the
 * sources registered above; u is that variable, u0..u3 the variables at the
 * same point (pamr_gb300.h). Variable 0's operator is the one registered by
 * amrd_set_device_MG_operator. solve_elliptics solves them together
 * (FP64 form); vcycle carries one variable. Returns 1, or 0 with a
 * message. */
int amrd_set_device_MG_var_operator(int var, char *lop, char *jac);

/* 0 (default): every operation in FP64, bit-identical to the reference;
 * 1: FP32 smoothing and prolongation inside FP64 defect correction
 * (pamr_gb300.h, PGB_MIXED). Returns 1, or 0 for another value. */
int amrd_set_device_MG_precision(int precision);

/* The finest-level residual after each V-cycle of the last solve_elliptics
 * (up to cap values); returns the number of cycles. */
int amrd_device_MG_residuals(double *res, int cap);

/* Frees the cached device hierarchy (it is rebuilt when the AMR hierarchy
 * changes anyway). */
void amrd_device_MG_release(void);

#ifdef __cplusplus
}
#endif
#endif
