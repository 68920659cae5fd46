/*
 * Device-side level descriptors and kernel launchers of libpamr_gb300.
 * The launchers are plain C entry points (extern "C") called by the C host
 * driver; every pointer argument is a device pointer.
 */
#ifndef PGB_DEV_H
#define PGB_DEV_H

#include "pgb_internal.h"

#ifdef __cplusplus
extern "C" {
#endif

/* tile extents: one CTA of 32 x 8 threads; each thread walks up to PGB_TZ
 * planes in 3-D (fewer on small levels, so they still spread over the
 * SMs). Relax tiles are twice as wide in x because a thread updates one
 * point of the active colour out of every two. */
#define PGB_TX 32
#define PGB_TY 8
#define PGB_TZ 8

/* one MG level as the kernels see it */
typedef struct {
   const pgb_tile *tiles;      /* 32 x 8 x TZ tiles over every box of the level */
   const pgb_tile *rtiles;     /* 64 x 8 x TZ tiles (relax) */
   const int *tile_start;      /* per level box: first tile (prefix, nbox+1) */
   const int *rtile_start;
   const int *box;             /* level box -> global box index */
   const pgb_tile *ctiles;     /* tiles holding a child-covered point or a point some
                                  interpolation to the next finer level reads */
   const pgb_tile *ztiles;     /* 32 x 8 x ztz columns (one-pass marching sweep, 3-D) */
   const pgb_tile *mtiles;     /* mtx x 14 x mtz columns (TMA-staged one-pass sweep, 3-D) */
   const void *tmaps;          /* its tensor maps (8 per box), or 0 where the level cannot use it */
   int *err;                   /* device word a timed-out wait of that sweep sets */
   int nmtiles, mtx, mtz;
   int ntiles, nrtiles, nbox, nctiles, nztiles;
   int tz, rtz, ztz;           /* planes per tile (3-D) of the tile lists */
   int dim;
   int level;
   int nvar;                   /* elliptic variables (1..PGB_NVAR_MAX) */
} pgb_dlevel;

/* device-side trace of every norm a hook would return (kind 0 relax,
 * 1 residual), one record per box and call; repeat > 1 marks coarsest-grid
 * iterations that were skipped because the iteration had reached a cycle */
typedef struct {
   int kind, level, box, repeat;
   double norm;
} pgb_trace_rec;

typedef struct {
   int n, cap, overflow, pad;
   pgb_trace_rec rec[1];
} pgb_trace;

/* scratch the reductions use (device memory) */
typedef struct {
   double *partial;            /* >= 2 * max tiles of any level */
   unsigned int *counter;      /* one word, zero between kernels */
   double *box_norm;           /* >= max boxes of any level */
   long npartial;              /* entries of partial */
} pgb_scratch;

/* parameters of the coarsest-grid loop (amrd/mg.c:172-190) */
typedef struct {
   int start_iter, max_citer;
   double crtol;
   const double *res_dn;       /* res[L] from the down sweep (ctol base) */
   double *res_out;            /* res[L] after the loop */
   int *iters_out;             /* iterations executed (for statistics) */
   int stagnation_exit;        /* mixed form: also stop when the norm stops decreasing */
   int ctol_from_first;        /* mixed form: ctol = crtol x the loop's first norm */
   long smem_points;           /* points of the level's coarsest boxes (on-chip kernel) */
   int ncoarse;                /* number of coarsest boxes on the level */
   double omega;               /* mixed form: over-relaxation factor of the loop */
   int sor;                    /* mixed form, several variables: the FP64 loop solves each point's
                                  variables together (Newton), over-relaxed by omega */
   int inner_sweeps;           /* mixed form: FP32 sweeps per FP64 defect correction */
   double *snap;               /* 2 x (points of the coarsest boxes) doubles */
   long snap_points;
   const long *snap_off;       /* per level box: offset of its points in a snapshot */
} pgb_coarsest_args;

const char *pgb_dev_error(void);
void pgb_note_error(const char *msg);   /* sets the message pgb_last_error returns */
unsigned long long pgb_dev_launches(void);
int pgb_dev_sync(void *stream);

/* FP64 path: every expression follows the reference hooks / Fortran order
 * and the file is compiled without FMA contraction */
int pgb_k_clear(const pgb_dbox *boxes, pgb_dlevel lv, int field_mask, void *stream);
int pgb_k_relax(const pgb_dbox *boxes, pgb_dlevel lv, int pde, pgb_scratch sc, double *norm_out,
                pgb_trace *trace, void *stream);
int pgb_k_residual(const pgb_dbox *boxes, pgb_dlevel lv, int pde, pgb_scratch sc,
                   double *norm_out, pgb_trace *trace, void *stream);
int pgb_k_lop_rhs(const pgb_dbox *boxes, pgb_dlevel lv, int pde, double w0_r, void *stream);
int pgb_k_cgc_coarse(const pgb_dbox *boxes, pgb_dlevel lv, double w0_i, void *stream);
int pgb_k_add_res(const pgb_dbox *boxes, pgb_dlevel lv, void *stream);
int pgb_k_copy(const pgb_dbox *boxes, const pgb_plan *p, int field, void *stream);
/* restricts the fields of field_mask (bit f = grid function f) that the plan's ops carry;
 * res32 = 1: the full weighting of res from the mixed form's FP32 copy of -res */
int pgb_k_restrict(const pgb_dbox *boxes, const pgb_plan *p, int field_mask, int res32, void *stream);
int pgb_k_interp(const pgb_dbox *boxes, const pgb_plan *p, int field, int dim, void *stream);
int pgb_k_coarsest(const pgb_dbox *boxes, pgb_dlevel lv, int pde, const pgb_plan *sync,
                   pgb_coarsest_args a, pgb_trace *trace, void *stream);
int pgb_k_fill(double *p, long n, double v, void *stream);

/* excision m_util_r8 kernels (pgb_mutil_ex.cu) */
unsigned long long pgb_dev_launches_ex(void);
unsigned long long pgb_dev_launches_net(void);   /* pgb_net.cu */
unsigned long long pgb_dev_launches_bo(void);    /* pgb_bo.cu */
unsigned long long pgb_dev_launches_diss(void);  /* pgb_diss.cu */
unsigned long long pgb_dev_launches_lb(void);    /* pgb_linbnd.cu */

/* mixed-precision path (pgb_kernels32.cu) */
const char *pgb_dev_error32(void);
unsigned long long pgb_dev_launches32(void);
int pgb_k_fas_defect(const pgb_dbox *boxes, pgb_dlevel lv, int pde, double w0_r, int cover, void *stream);
/* D -= lap E + C E at relaxed points; with gate, only while *gate == gval */
int pgb_k_defect32(const pgb_dbox *boxes, pgb_dlevel lv, int slot, const int *gate, int gval, void *stream);
int pgb_k_flip(int *parity, void *stream);
int pgb_k_sweep32(const pgb_dbox *boxes, pgb_dlevel lv, int nsweep, int fuse, int *slot, void *stream);
/* tensor maps of the TMA-staged sweep (8 per box); 0, or 1 where unavailable */
int pgb_tmaps_build(const pgb_dbox *hbox, int nbox, void **d_maps);
/* the device solve loop's step: records the finest norm of cycle *it,
 * counts the cycle and sets the while node's condition to pgb_solve's loop
 * test ((it < min_iter || res > tol) && it < max_iter) */
int pgb_k_solve_step(unsigned long long handle, const double *norm, double *hist, int *it, int min_iter,
                     int max_iter, double tol, void *stream);
int pgb_k_update(const pgb_dbox *boxes, pgb_dlevel lv, int post, int slot, int zslot, void *stream);
/* pgb_k_defect32 (defect = 1, gated like it) and pgb_k_update in one pass;
 * zslot must differ from slot */
int pgb_k_update_defect(const pgb_dbox *boxes, pgb_dlevel lv, int post, int slot, int zslot, int defect,
                        const int *gate, int gval, void *stream);
int pgb_k_zero32(const pgb_dbox *boxes, pgb_dlevel lv, void *stream);
int pgb_k_copy32(const pgb_dbox *boxes, const pgb_plan *p, int slot, void *stream);
int pgb_k_cgc_mixed(const pgb_dbox *boxes, pgb_dlevel lv, double inv_w0, void *stream);
int pgb_k_interp_mixed(const pgb_dbox *boxes, const pgb_plan *p, int dim, int slot, void *stream, void *side,
                       void *fork, void *join);
int pgb_k_residual_fast(const pgb_dbox *boxes, pgb_dlevel lv, int pde, pgb_scratch sc,
                        double *norm_out, pgb_trace *trace, const int *gate, void *stream);
int pgb_k_lop_rhs_fast(const pgb_dbox *boxes, pgb_dlevel lv, int pde, double w0_r, void *stream);
/* the box tables of the variables of a mixed-form solve with several
 * elliptic variables: t[v] is variable v's view (t[0] the solver's table) */
typedef struct {
   const pgb_dbox *t[PGB_NVAR_MAX];
} pgb_vtabs;
/* the coupling coefficients of the view's variable on a level, where they
 * do not depend on the state (pgb_dop.cfixed; the passes skip them then) */
int pgb_k_couplings(const pgb_dbox *boxes, pgb_dlevel lv, void *stream);
/* one colour pass of the coupled FP32 smoother over lv.nvar variables */
int pgb_k_relax32_vars(pgb_vtabs vt, pgb_dlevel lv, int pass, void *stream);
/* the level's norm over the res of every elliptic variable (lv.nvar of them) */
int pgb_k_norm_vars(const pgb_dbox *boxes, pgb_dlevel lv, pgb_scratch sc, double *norm_out, pgb_trace *trace,
                    void *stream);
int pgb_k_coarsest_mixed(const pgb_dbox *boxes, pgb_dlevel lv, int pde, const pgb_plan *sync,
                         pgb_coarsest_args a, pgb_trace *trace, void *stream);

/* The small-level kernel (mixed form). The V-cycle's passes over its small
 * levels (residual, restriction, FAS right-hand side, colour passes, defect
 * carry and update, coarsest-grid loop, coarse-grid correction and
 * interpolation) are recorded, not launched, while recording is on: each
 * launcher above appends a step with its arguments and launch geometry.
 * pgb_k_tail then runs every step in one launch of one thread-block
 * cluster, the cluster's CTAs sharing each step's blocks and meeting at a
 * cluster barrier between steps. The program travels as the kernel's
 * parameter (it stays in the launch, or in the graph node that captured
 * it). Each step runs the body of the kernel it replaces, so every value is
 * the same bit for bit. */
#define PGB_TAIL_MAXLEV 8
#define PGB_TAIL_MAXSTEP 224
typedef struct {
   unsigned char kind, lev, bar, solo;  /* step kind, index into lv[], barrier after it (0 none,
                                           1 the cluster's, 2 CTA 0's), run by CTA 0 alone */
   int a[6];                            /* integer arguments of the kernel it replaces */
   int gx, gy, gz;                      /* that kernel's grid */
   const void *ptr;                     /* op list or gate */
   double d;                            /* w0_r or 1/w0_i */
} pgb_tail_step;

typedef struct {
   int nstep, nlev, pde, ncsync;
   size_t smem;                         /* dynamic shared memory (the coarsest-grid loop) */
   size_t prog_off;                     /* where the kernel keeps its copy of this program in shared
                                           memory (after the coarsest loop's), 0: read in place */
   size_t smem_total;                   /* dynamic shared memory of the launch */
   int nbox_copy;                       /* boxes of the box table copied to shared memory (0: none) */
   int grid;                            /* 0: one cluster (hardware barrier); 1: one CTA per SM in a
                                           cooperative launch, meeting at a counter in global memory */
   unsigned int *bar_cnt;               /* that counter (zeroed before each launch) */
   int *err;                            /* set to 4 when a wait at it runs out (about 0.5 s) */
   int mini;                            /* 1: one CTA, the levels' arrays staged in shared memory */
   int nbox_all;                        /* boxes of the whole box table (copied when mini) */
   size_t mini_off;                     /* where the staged arrays start in shared memory */
   pgb_dlevel lv[PGB_TAIL_MAXLEV];
   pgb_coarsest_args ca;                /* the coarsest-grid loop's arguments */
   const pgb_copy_op *csync;            /* and its sync ops */
   pgb_tail_step step[PGB_TAIL_MAXSTEP];
} pgb_tail_prog;

/* mini_bytes > 0: mini mode, the program's levels' arrays (that many bytes)
 * staged in the shared memory of one CTA */
void pgb_tail_begin(pgb_tail_prog *p, int pde, int nbox, size_t mini_bytes);
/* steps recorded from now on run in CTA 0 alone (levels so small that one
 * CTA's L1 holds them: consecutive such steps meet at a CTA barrier) */
void pgb_tail_set_solo(int on);
/* stops recording; 1 when a pass could not be recorded (pgb_dev_error32 says which) */
int pgb_tail_end(void);
int pgb_tail_recording(void);
/* the FP64-file passes (pgb_kernels64.cu) while recording */
int pgb_tail_add_restrict(const pgb_plan *p, int field_mask, int res32);
int pgb_tail_add_clear(pgb_dlevel lv, int mask);
/* runs a recorded program on a cluster of ncta CTAs */
int pgb_k_tail(const pgb_dbox *boxes, const pgb_tail_prog *p, int ncta, pgb_scratch sc, void *stream);
/* CTAs of a launch in grid mode: one per SM */
int pgb_tail_grid_ctas(void);
/* the largest cluster (16, 8, 4, 2 or 1 CTAs) the device schedules for the
 * small-level kernel with smem bytes of dynamic shared memory; 0 if none */
int pgb_tail_max_cluster(size_t smem);

#ifdef __cplusplus
}
#endif
#endif
