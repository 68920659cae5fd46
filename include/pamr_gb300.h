/*
 * pamr_gb300.h --- C ABI of libpamr_gb300, a GB300 (sm_103a) implementation
 * of AMRD's FAS multigrid elliptic solve and the PAMR grid-function
 * transfers it uses.
 *
 * Plain C: opaque handles, plain pointers and sizes, int status codes (0 =
 * success; on failure pgb_last_error() describes the problem). Nothing here
 * exits the process (the reference's AMRD_stop, amrd/util.c:27-34, does).
 *
 * Each entry point names the reference interface it replaces
 * (paths relative to the reference project).
 */
#ifndef PAMR_GB300_H
#define PAMR_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* PDE kinds of the device-side level operators; the operator is
 * L[u] = lap(u) + term, evaluated as the reference hook pattern
 * examples/nbs/num.f:85-246 does:
 *   PGB_PDE_POISSON   term = -src               (lap u = rho)
 *   PGB_PDE_CONFORMAL term = +2 pi src u^5       (conformal factor)
 *   PGB_PDE_LAPSE     term = -src u              (maximal-slicing lapse) */
#define PGB_PDE_POISSON 0
#define PGB_PDE_CONFORMAL 1
#define PGB_PDE_LAPSE 2

/* transfer operators (PAMR transfer bits, include/pamr.h:92-105) */
#define PGB_STRAIGHT_INJECT 1
#define PGB_HW_RESTR 2
#define PGB_FW_RESTR 3

/* pgb_create flags */
#define PGB_HOST_ONLY 1      /* build hierarchy and transfer plans only (no GPU) */

/* Multigrid parameters: the AMRD run-time knobs (amrd/io.c:96-109, 269-288,
 * doc/AMRD_ref.tex:575-631) plus the per-variable transfer operators of
 * the parameter lists mg_hw_restr / mg_fw_restr / mg_interp2. */
typedef struct {
   int pre_swp, pst_swp;        /* MG_pre_swp, MG_pst_swp */
   int max_iter, min_iter;      /* MG_max_iter, MG_min_iter */
   int max_citer;               /* MG_max_citer */
   double tol;                  /* MG_tol (absolute, finest-level residual norm) */
   double crtol;                /* MG_crtol */
   double w0_r, w0_i;           /* MG_w0_r, MG_w0_i */
   int min_cwidth;              /* min_mg_cwidth */
   int restr_u, restr_res, restr_src;  /* restriction of u, u_res, source */
   int interp_order;            /* 2 (mg_interp2) or 4 */
   int interp_buffer;           /* PAMR interp_buffer, default 2 (src/pamr.c:157) */
   int precision;               /* PGB_FP64 (bit-exact with the reference) or PGB_MIXED */
} pgb_mg_params;

/* precision of pgb_mg_params:
 *   PGB_FP64  every operation in FP64, results bit-identical to the reference
 *   PGB_MIXED FP32 smoothing (Gauss-Seidel on the correction of each smoothing
 *             block) and FP32 prolongation inside FP64 defect correction;
 *             residuals, restriction, FAS right-hand sides, coarsest-grid
 *             solve and solution updates stay FP64 */
#define PGB_FP64 0
#define PGB_MIXED 1

typedef struct pgb_solver pgb_solver;

/* Last error message of the calling thread. */
const char *pgb_last_error(void);

/* Default parameters (AMRD defaults, V(2,2), tol 0). */
void pgb_default_params(pgb_mg_params *p);

/* Builds the AMR hierarchy from `ngrids` grids (level grid_level[i] >= 1,
 * bounding box grid_bbox[6*i .. 6*i+5] = x0,x1,y0,y1,z0,z1), the MG
 * hierarchy below/among it, every transfer plan, and (unless
 * PGB_HOST_ONLY) the device arena on the current CUDA device.
 * Replaces PAMR_compose_hierarchy (src/pamr.c:259) followed by
 * PAMR_build_mgh (src/pamr.c:354, src/gh.c:1222); refinement ratio 2. */
int pgb_create(int dim, int pde, const int *base_shape, const double *base_bbox, int ngrids,
               const int *grid_level, const double *grid_bbox, const pgb_mg_params *params,
               int flags, pgb_solver **out);

/* ------------------------------------------------------ level operators -- */
/* An elliptic operator for the device, registered by the application
 * (additive: the reference keeps its operator in the host hooks
 * app_L_op / app_MG_residual / app_MG_relax, include/amrd.h:137-159, which
 * run per grid on host arrays; the GPU needs the same arithmetic on the
 * device). The operator is two expressions:
 *   lop  L[u]  of lap, u, s0..s<nsrc-1> and numbers, e.g. "lap - s0"
 *   jac  dL/du of j0, u, s0.. and numbers,           e.g. "j0"
 * lap is the 5-point (2-D) / 7-point (3-D) Laplacian of u written as the
 * reference hooks form it, ((u+ - 2u + u-)/dx^2 + (..)/dy^2) + (..)/dz^2
 * (examples/nbs/num.f:113-115); j0 = -2/dx^2 - 2/dy^2 [- 2/dz^2]
 * (num.f:236); sK is the K-th source grid function at the point. +, -, *,
 * / and unary minus with parentheses; equal precedence associates to the
 * left and every operation rounds once in IEEE double, so an expression in
 * the hook's order gives the hook's results bit for bit (nbs:
 * "lap - (s0*s0 + s1*s1)", "j0"). Relaxation updates
 * u <- u - (L[u] - rhs) / (dL/du) at each red, then black point
 * (num.f:216-241). A solver with several elliptic variables takes one
 * operator per variable: u is the equation's own variable and u0..u3 the
 * variables' values at the same point; relaxation updates the variables
 * in order at each point, each from the others' current values. At most PGB_MAX_SOURCES sources, 31 operations and 8
 * distinct constants per expression. */
#define PGB_MAX_SOURCES 4
#define PGB_MAX_VARS 4
typedef struct pgb_operator pgb_operator;
int pgb_operator_create(int nsrc, const char *lop, const char *jac, pgb_operator **out);
/* the built-in operators PGB_PDE_* as operator objects */
int pgb_operator_builtin(int pde, pgb_operator **out);
void pgb_operator_destroy(pgb_operator *op);
int pgb_operator_nsrc(const pgb_operator *op);
/* PGB_PDE_* when the program is one of the built-in operators (evaluated
 * by compiled code, same arithmetic), 3 for any other program */
int pgb_operator_kind(const pgb_operator *op);
/* The operator at one point on the host, with the device's rounding: L[u]
 * and dL/du from lap, j0, u and the source values s[0..nsrc-1] (either of
 * L, J may be NULL). Lets host code (an application's own hooks on host
 * copies of its grids) evaluate exactly what the device evaluates. */
int pgb_operator_eval(const pgb_operator *op, double lap, double j0, double u, const double *s, double *L,
                      double *J);
/* the same with several elliptic variables: the value of every variable at
 * the point in uv[0..3] (u0..u3), var the equation's own variable (u) */
int pgb_operator_eval_vars(const pgb_operator *op, int var, double lapv, double j0, const double *uv,
                           const double *s, double *L, double *J);
/* 1 + the highest variable index the operator names (u0..u3), 0 if none */
int pgb_operator_vars(const pgb_operator *op);

/* Everything pgb_create takes, plus the level operator, the coarsest AMR
 * level of the MG hierarchy (min_level: PAMR_build_mgh(min_lev, max_lev, tl),
 * src/gh.c:1222; grids below it are ignored and the MG levels below it are
 * coarsenings of its grids; amrd/mg.c:29 builds from the level
 * solve_elliptics is given, amrd/evolve.c:454 from the finest alone) and
 * the MG restriction of each source (restr_src[0] is params.restr_src). */
typedef struct {
   int dim;
   const pgb_operator *op;      /* copied at creation */
   int base_shape[3];
   double base_bbox[6];
   int ngrids;
   const int *grid_level;
   const double *grid_bbox;
   pgb_mg_params params;
   int min_level;               /* 1 = the whole AMR hierarchy */
   int restr_src[PGB_MAX_SOURCES];
   int flags;
   /* several elliptic variables solved together (AMRD_num_elliptic_vars,
    * amrd/mg.c:248-314): nvar (1..PGB_MAX_VARS) and the operator of each
    * variable v >= 1 in var_op[v] (op is variable 0's); both forms (the
    * mixed form smooths all variables' FP32 corrections point by point, with
    * coupling coefficients from the programs' derivatives). Every variable
    * takes the same transfer operators (restr_u, restr_res, mg_sync,
    * interp_order) */
   int nvar;
   const pgb_operator *var_op[PGB_MAX_VARS];
} pgb_create_args;
void pgb_default_create_args(pgb_create_args *a);
int pgb_create_ex(const pgb_create_args *a, pgb_solver **out);

/* Frees the hierarchy and device memory (PAMR_destroy_mgh, src/pamr.c:383). */
int pgb_destroy(pgb_solver *s);

/* Grid data. Arrays are float64, x fastest (Fortran u(Nx,Ny,Nz)), shape
 * from pgb_grid_shape. Host-pointer variants copy through the solver's
 * stream; the *_device variants take device pointers. These replace the
 * raw gfs pointers applications read via PAMR_get_g_attribs
 * (src/pamr.c:1706) for the elliptic variable and its source. */
int pgb_grid_shape(const pgb_solver *s, int grid, int *shape3);
int pgb_set_grid(pgb_solver *s, int grid, const double *u, const double *src);
int pgb_get_grid(pgb_solver *s, int grid, double *u);
int pgb_set_grid_device(pgb_solver *s, int grid, const double *u, const double *src);
int pgb_get_grid_device(pgb_solver *s, int grid, double *u);
/* source k (0 <= k < the operator's source count) of an input grid;
 * pgb_set_grid's src is source 0 */
int pgb_set_source(pgb_solver *s, int grid, int k, const double *src);
int pgb_set_source_device(pgb_solver *s, int grid, int k, const double *src);
/* elliptic variable v (0 <= v < nvar) of an input grid; v = 0 is the u of
 * pgb_set_grid / pgb_get_grid */
int pgb_set_var(pgb_solver *s, int grid, int v, const double *u);
int pgb_get_var(pgb_solver *s, int grid, int v, double *u);

/* Full solve: rebuilds the MG-only data from the AMR grids (build_mgh's
 * injections), then V-cycles until the finest residual is <= tol (at least
 * min_iter, at most max_iter cycles). Replaces solve_elliptics
 * (amrd/mg.c:20-79). res_per_cycle (may be NULL) receives up to cap
 * residuals. The cycles and the stopping test run on the device (one CUDA
 * graph with a conditional while node; the host waits once per solve);
 * environment PGB_HOST_LOOP=1 tests on the host after every cycle instead,
 * with the same results bit for bit. */
int pgb_solve(pgb_solver *s, int *iters, double *res_final, double *res_per_cycle, int cap);

/* One FAS V-cycle; *res = finest-level residual. Replaces vcycle
 * (amrd/mg.c:84-201). pgb_prepare performs the MG-hierarchy initialisation
 * pgb_solve does before its first cycle; pgb_vcycle runs it itself when an
 * input grid was set (pgb_set_grid*) or a level was swept by pgb_time_relax
 * since the last pgb_prepare. */
int pgb_prepare(pgb_solver *s);
int pgb_vcycle(pgb_solver *s, double *res);
/* pgb_prepare with flags: PGB_PREPARE_KEEP_MG_DATA leaves u of the pure MG
 * levels as stored with pgb_box_set instead of injecting it from the AMR
 * levels (an MG hierarchy that already exists, as PAMR keeps it between the
 * vcycle calls of amrd/evolve.c:471-487); their sources are injected from
 * the level above, as the reference's vcycle does in its down sweep
 * (src/pamr.c:677-680), so sources changed on the AMR levels since the
 * hierarchy was built reach them */
#define PGB_PREPARE_KEEP_MG_DATA 1
int pgb_prepare_ex(pgb_solver *s, int flags);

/* Grid functions of one box of the MG hierarchy (level, index in PAMR
 * grid-list order, as pgb_box_info), host arrays: PGB_FIELD_U the elliptic
 * variable f, _RES f_res, _LOP f_lop, _RHS f_rhs, PGB_FIELD_SRC + k
 * source k -- the MG-hierarchy gfs of PAMR_get_g_attribs with
 * PAMR_get_gfn(name, PAMR_MGH, 0) (src/pamr.c:1706-1762). Setting a box
 * makes the next pgb_vcycle start with pgb_prepare (use pgb_prepare_ex
 * first to keep MG-level data). */
#define PGB_FIELD_U 0
#define PGB_FIELD_RES 1
#define PGB_FIELD_LOP 2
#define PGB_FIELD_RHS 3
#define PGB_FIELD_SRC 4
/* the U..RHS fields of elliptic variable v >= 1: PGB_FIELD_VAR(v) + PGB_FIELD_U..RHS */
#define PGB_FIELD_VAR(v) (16 + 4 * ((v) - 1))
int pgb_box_set(pgb_solver *s, int level, int idx, int field, const double *in);
int pgb_box_get(pgb_solver *s, int level, int idx, int field, double *out);

/* The solver's CUDA stream (cudaStream_t) for callers that order their own
 * work around it. */
void *pgb_stream(pgb_solver *s);

/* Statistics of the last pgb_solve: V-cycles, coarsest-grid iterations
 * (as the reference counts them), and device time in ms. */
int pgb_stats(const pgb_solver *s, int *vcycles, long *coarsest_iters, double *device_ms);

/* Interpolation of u on the AMR hierarchy from AMR level lc to lc+1:
 * amr_bdy_width = 0 replaces PAMR_interp(lc, tl, PAMR_AMRH) (src/pamr.c:623),
 * the whole overlap; amr_bdy_width > 0 replaces PAMR_AMR_bdy_interp(lc, tl,
 * width) (src/pamr.c:645), the band of that width along the fine grids'
 * AMR boundaries. order 2 or 4 (the variable's amr_interp order); same
 * transfer lists and dminterp3d arithmetic as the reference, bit-exact. */
int pgb_amr_interp(pgb_solver *s, int lc, int amr_bdy_width, int order);

/* Regrid: replaces the data transfer of PAMR_compose_hierarchy onto a new
 * hierarchy (init_new_cgh, src/gh.c:934-1045, called at src/pamr.c:311).
 * dst is a solver created on the hierarchy after the regrid, src the solver
 * of the hierarchy it replaces (same dimension and source count). For every
 * AMR level L of dst, coarse to fine: if L >= min_level (the first level the
 * reference recomposes), u and the sources are interpolated (order 2 or 4,
 * the variables' regrid_transfer order) from src's level L-1 over dst's
 * whole level L; then on every level they are copied from src's grids of
 * level L where they overlap dst's. Same transfer lists and dminterp3d /
 * dmcopy3d arithmetic as the reference, bit-exact. Points of dst that
 * neither transfer reaches keep their values. Both solvers stay usable. */
int pgb_regrid(pgb_solver *dst, pgb_solver *src, int order, int min_level);

/* Checkpoint and restart of the device hierarchy's elliptic data (no
 * counterpart format in the reference, whose checkpoints are SDF files of
 * every grid function written through bbhutil, src/pamr.c:1908-1978,
 * 2042-2075): pgb_checkpoint_save writes, per input grid, its level, shape,
 * bounding box, u of every elliptic variable and the sources to `path`;
 * pgb_checkpoint_load restores them
 * into a solver created on the same hierarchy (checked bit for bit) and
 * fails without changing it when the file does not match. */
int pgb_checkpoint_save(pgb_solver *s, const char *path);
int pgb_checkpoint_load(pgb_solver *s, const char *path);

/* Kernel launches this library has issued in the process (all solvers). */
long long pgb_launch_count(void);

/* Times `reps` red-black relax sweeps (both colours, app_MG_relax on every
 * box, examples/nbs/num.f:172-246) of MG level `level` on the solver's
 * current data with CUDA events on its stream; returns the mean time per
 * sweep and the algorithmic bytes of one sweep: FP64 path 32 bytes per
 * interior point (u read and written, rhs and source read), mixed form 16
 * (FP32 correction read and written, defect and Jacobian term read).
 * The mixed form times its sweeps as a smoothing block of the V-cycle runs
 * them (blocks of MG_pre_swp sweeps with the level's tuned tile depth and
 * sweeps per launch; the autotuner runs first if it has not). Modifies u
 * (FP64) or the correction (mixed) on that level. */
int pgb_time_relax(pgb_solver *s, int level, int reps, double *ms_per_sweep,
                   double *bytes_per_sweep);

/* Launch shapes the mixed form's autotuner chose for a level at the first
 * pgb_prepare: tile depth in planes, and the FP32 sweep kernel (0 = one
 * launch per colour pass, 1 or 2 = sweeps per launch staged in shared
 * memory, 3 = one sweep per launch in one pass over memory, marching
 * through the tile's planes, 4 or 5 = one sweep per launch with planes
 * staged by TMA in columns 60 or 28 points wide, 6 or 7 = two sweeps per
 * launch staged by TMA in columns 24 or 56 points wide; 3-7 on 3-D levels
 * only; a solver with several elliptic variables runs the coupled colour
 * passes and reports 0); no reference counterpart. */
int pgb_level_tuning(pgb_solver *s, int level, int *tile_planes, int *sweeps_per_launch);

/* Mixed form: MG levels 1..n (the return value; 0 when none) whose V-cycle
 * passes run as one launch of the small-level kernel, a thread-block
 * cluster of *cluster_ctas CTAs (levels of at most PGB_TAIL_POINTS points,
 * 6000 unless set). Off unless the environment sets PGB_TAIL=1 (or
 * PGB_TAIL=mini: one CTA, the levels' arrays in its shared memory, levels of
 * at most 1500 points); it gives the same bits and was measured slower than
 * one launch per pass on GB300. pgb_level_tuning reports sweep mode 8 for
 * those levels. Known
 * after the first pgb_prepare. No reference counterpart (the reference
 * relaxes grid by grid on the host). */
int pgb_tail_levels(const pgb_solver *s, int *cluster_ctas);

/* Norm trace: when enabled, every norm a hook would return is recorded
 * (kind 0 relax, 1 residual, 2 = skipped coarsest iterations; level; box;
 * repeat; norm) -- the device counterpart of MG_trace (amrd/mg.c:138-195). */
int pgb_trace_enable(pgb_solver *s, int capacity);
int pgb_trace_fetch(pgb_solver *s, int *kind, int *level, int *box, int *repeat, double *norm,
                    int cap, int *n);

/* ---------------------------------------------------- hierarchy queries -- */
int pgb_num_levels(const pgb_solver *s);
int pgb_level_nbox(const pgb_solver *s, int level);
/* box `idx` of MG level `level` in PAMR grid-list order */
int pgb_box_info(const pgb_solver *s, int level, int idx, int *shape3, double *bbox6,
                 int *coarsest, int *amr_grid);
/* cmask arrays: kind 0 = set_cmask_bdy (amrd/mg.c:432), 1 = set_cmask_child
 * (amrd/mg.c:362); values 1.0 (AMRD_CMASK_ON) / 0.0 */
int pgb_box_cmask(const pgb_solver *s, int level, int idx, int kind, double *out);
/* transfer plans as index rows (which: 0 sync bw0, 1 sync bw1, 2 sync
 * coarsest, 3 inject, 4 inject at build, 5 interp); returns the op count
 * and fills up to cap rows of 24 ints */
int pgb_plan_dump(const pgb_solver *s, int which, int level, int *rows, int cap);

/* ------------------------------------------- residual without allocation -- */
/* No counterpart in the reference. The residual of ONE grid,
 * res = L[u] - rhs at interior points where cmask is ON (cmask = NULL: all
 * interior points), and its RMS norm written to *norm (device double), as
 * app_MG_residual computes them. cmask is one byte per point, nonzero =
 * AMRD_CMASK_ON (PAMR keeps cmask as doubles 1.0 / 0.0: convert); points
 * where it is 0 and the grid's boundary points are not written. With no ON
 * point the norm is 0/0, NaN, as the reference hook's sqrt(norm/sum)
 * (examples/nbs/num.f:158). For callers that cannot allocate device
 * memory when they need it: applications that own and budget all device
 * memory themselves (as PAMR owns all grid memory), and callers that must
 * not let a cudaMalloc/cudaFree synchronize the device between their
 * asynchronous launches. All pointers except shape3/dx3 (host) are device
 * pointers supplied by the caller; the reduction uses a fixed 64 KiB array
 * in device global memory that every GPU loading the library holds until
 * process exit. Limit: the grid must fit in PGB_NOALLOC_MAX_TILES tiles of
 * 32 x 8 x 8 points (ceil(Nx/32)*ceil(Ny/8)*ceil(Nz/8), Nz term 1 in 2-D;
 * e.g. 161^3 or 1000 x 1000). The first call on a device looks up the
 * array's device address; make it before any stream capture. Calls share
 * the array: calls whose kernels overlap on the GPU race and must not be
 * issued that way. Returns 0, or 1 bad arguments, 2 grid above the limit,
 * 3 no device / address lookup failed, 4 launch failed (a message is
 * printed on stderr). Allocates nothing. */
#define PGB_NOALLOC_MAX_TILES 4095
int pgb_residual_norm_noalloc(int pde, int dim, const int *shape3, const double *dx3,
                              const double *u, const double *rhs, const double *src,
                              const unsigned char *cmask, double *res, double *norm,
                              void *stream);

/* --------------------------------- device m_util_r8 (include/m_util_r8.h) -- */
/* Same arguments as the Fortran routines (src/m_util_r8.f), by value, on
 * device arrays; stream may be NULL. No excision (do_ex = 0). */
int pgb_dmcopy3d(const double *u1, double *u2, int nx1, int ny1, int nz1, int nx2, int ny2,
                 int nz2, int i1, int j1, int k1, int i2, int j2, int k2, int ni, int nj, int nk,
                 int si1, int sj1, int sk1, int si2, int sj2, int sk2, void *stream);
int pgb_dmhwr3d(const double *u1, double *u2, int nx1, int ny1, int nz1, int nx2, int ny2,
                int nz2, int i1, int j1, int k1, int i2, int j2, int k2, int ni, int nj, int nk,
                int si1, int sj1, int sk1, int si2, int sj2, int sk2, void *stream);
int pgb_dmfwr3d(const double *u1, double *u2, int nx1, int ny1, int nz1, int nx2, int ny2,
                int nz2, int i1, int j1, int k1, int i2, int j2, int k2, int ni, int nj, int nk,
                int si1, int sj1, int sk1, int si2, int sj2, int sk2, void *stream);
int pgb_dminterp3d(const double *u1, double *u2, int nx1, int ny1, int nz1, int nx2, int ny2,
                   int nz2, int i1, int j1, int k1, int i2, int j2, int k2, int ni, int nj,
                   int nk, int si1, int sj1, int sk1, int irho, int jrho, int krho, int ord,
                   void *stream);

/* Excision variants (do_ex = 1 in the Fortran): chr1 is the mask of u1 on
 * the device (a point is excised where chr1 == ex). dmhwr3d_ex and
 * dmfwr3d_ex replace dmhwr3d/dmfwr3d(..., chr1, ex, 1) (src/m_util_r8.f:
 * 649-723, 733-949); dminterp3d_ex replaces dminterp3d(..., chr1, ex, 1)
 * (src/m_util_r8.f:473-637 with dvi2q1d_ex/dvi4q1d_ex) and, like it,
 * overwrites parts of u2's excised zone. */
int pgb_dmhwr3d_ex(const double *u1, double *u2, int nx1, int ny1, int nz1, int nx2, int ny2,
                   int nz2, int i1, int j1, int k1, int i2, int j2, int k2, int ni, int nj, int nk,
                   int si1, int sj1, int sk1, int si2, int sj2, int sk2, const double *chr1,
                   double ex, void *stream);
int pgb_dmfwr3d_ex(const double *u1, double *u2, int nx1, int ny1, int nz1, int nx2, int ny2,
                   int nz2, int i1, int j1, int k1, int i2, int j2, int k2, int ni, int nj, int nk,
                   int si1, int sj1, int sk1, int si2, int sj2, int sk2, const double *chr1,
                   double ex, void *stream);
int pgb_dminterp3d_ex(const double *u1, double *u2, int nx1, int ny1, int nz1, int nx2, int ny2,
                      int nz2, int i1, int j1, int k1, int i2, int j2, int k2, int ni, int nj,
                      int nk, int si1, int sj1, int sk1, int irho, int jrho, int krho, int ord,
                      const double *chr1, double ex, void *stream);

/* ------------------------------------------------- learned initial guess -- */
/* No reference counterpart. BF16 tensor-core 3x3x3 convolution (tcgen05,
 * FP32 accumulation) on the channel-blocked, zero-padded activation layout
 * of the learned initial guess: act[cb][vtot][8] BF16 for channel block cb
 * (8 channels), voxel (x,y,z) of a W x H x D volume at index
 * margin + (x+1) + (W+2)*((y+1) + (H+2)*(z+1)); everything else zero.
 * pgb_conv3d_geometry returns vtot and margin; pgb_conv3d_pack_weights turns
 * FP32 weights w[27][cin][cout] (tap = dz*9 + dy*3 + dx) into the kernel's
 * BF16 image (adjoint = 1: the image of the transposed convolution, with
 * cin and cout exchanged); pgb_conv3d_bf16 computes
 * out = [act](conv(in) + bias) (bias may be NULL; act, applied when
 * relu = 1, is leaky ReLU with negative slope 1/8), writing zero on the
 * padding. Channel counts 16, 32 or 64; any volume of at least one
 * voxel (the margins absorb the over-reach of the last 128-voxel tile on
 * small volumes). err (device int, may be
 * NULL) is set when a wait inside the kernel runs out. */
int pgb_conv3d_geometry(int W, int H, int D, long *vtot, long *margin);
int pgb_conv3d_pack_weights(const float *w, void *img, int cin, int cout, int adjoint, void *stream);
int pgb_conv3d_bf16(const void *in, void *out, const void *wimg, const float *bias, int W, int H, int D,
                    int cin, int cout, int relu, int *err, void *stream);

/* Kreiss-Oliger dissipation, dmdiss3d (src/m_util_r8.f:1690-1956;
 * include/m_util_r8.h:33-36), on device arrays f, work, eps (eps[0] is the
 * coefficient, as eps(1,1,1)), mask; phys_bdy_type is a host array of 6.
 * Bit-exact with the Fortran, including the excised path (do_ex != 0,
 * dmdiss3d_ex, src/m_util_r8.f:972-1332: chr a device mask, eps per point
 * when do_ex < 0), where stencils that would leave the array in the
 * Fortran are skipped. Called by AMRD after each step on the dissipated
 * variables (amrd/evolve.c:430, 509, 957). */
int pgb_dmdiss3d(double *f, double *work, const double *eps, int do_bdy, const int *phys_bdy_type,
                 int even, int odd, const double *mask, double mask_off, int nx, int ny, int nz,
                 const double *chr, double ex, int do_ex, void *stream);

/* Linear approach to the boundaries, linbnd3d (src/m_util_r8.f:1957-2252;
 * include/m_util_r8.h:38-39) on a device array f (chr: device mask when
 * do_ex != 0); phys_bdy is a host array of 6 (1 physical, 0 AMR);
 * which_bnd 1 physical, 2 AMR, 3 both. Bit-exact with the Fortran; the
 * invalid extents the Fortran stops on return an error, and so does
 * Ny = 1 with Nz > 1, where the Fortran indexes outside f. */
int pgb_linbnd3d(double *f, const int *phys_bdy, int which_bnd, int Nx, int Ny, int Nz,
                 const double *chr, double ex, int do_ex, void *stream);

/* Berger-Oliger bookkeeping of the elliptic variables on the device, for
 * an application that keeps them there across coarse steps. Grids are host
 * arrays of device pointers with their AMR levels (level[g]) and point
 * counts (n[g]); all work is queued on `stream`.
 * pgb_mg_extrap: the new-time-level guess of one grid on a level > 1
 *   (amrd/evolve.c:344-366): method 0 (AMRD_MG_EXTRAP_2ND_FROM_ETM1)
 *   mgf0 = f1 etm1 + f2 etm2 with f1, f2 from tnp1, the parent's tnp1_lm1
 *   and dt_lm1; method 1 (AMRD_MG_EXTRAP_2ND_FROM_TN)
 *   mgf0 = mgf1 + dt/dt_lm1 (etm2 - etm1).
 * pgb_update_mg_extrap_vars: update_mg_extrap_vars (amrd/evolve.c:1640-1700):
 *   etm1 -> etm2, mgf1 -> etm1, and on levels > 1 with eps_c != 0
 *   etm2 += (etm1 - brs)(1 - eps_c/net_rho); rho_tm as PAMR_get_rho returns it.
 * pgb_set_mg_brs_vars: set_mg_brs_vars (amrd/evolve.c:1621-1638), brs = mgf1
 *   on levels L1..L2.
 * Bit-exact with the reference's loops. */
int pgb_mg_extrap(int method, double tnp1, double tnp1_lm1, double dt, double dt_lm1, double *mgf0,
                  const double *mgf1, const double *etm1, const double *etm2, long n, void *stream);
int pgb_update_mg_extrap_vars(int L1, int Lf, const int *rho_tm, int ngrids, const int *level,
                              double *const *etm1, double *const *etm2, const double *const *mgf1,
                              const double *const *brs, const long *n, double eps_c, void *stream);
int pgb_set_mg_brs_vars(int L1, int L2, int ngrids, const int *level, double *const *brs,
                        const double *const *mgf1, const long *n, void *stream);

/* The learned initial guess: a 6-level convolutional encoder-decoder
 * (16/32/64/64/64/64 channels, levels halving down to (n-1)/32 points a
 * side, two 3x3x3 convolutions per encoder level, one per decoder level,
 * additive skips, leaky ReLU) from a source rho on an n^3 grid (points 0..n-2
 * seen by the net; n-1 a multiple of 32, 65 <= n <= 513) to a guess of u, zero on
 * the grid boundary. Forward and backward-data convolutions of the inner
 * sixteen layers run on the tensor cores (BF16, FP32
 * accumulation); weight gradients and the 1-channel first and last layers
 * on CUDA cores; Adam on FP32 master weights. rho and u are device n^3
 * arrays (x fastest); the training target is FP32. Scales: the net reads
 * s_in * rho and predicts u / s_out. */
typedef struct pgb_net pgb_net;
int pgb_net_create(int n, unsigned long long seed, pgb_net **out);
void pgb_net_destroy(pgb_net *net);
int pgb_net_set_scales(pgb_net *net, double s_in, double s_out);
long pgb_net_num_params(pgb_net *net);
/* on = 1: all biases held at zero (cleared now, not trained), making the
 * net positively homogeneous, net(c rho) = c net(rho) for c > 0 -- the
 * right form for a guess of a linear equation's solution */
int pgb_net_set_bias_free(pgb_net *net, int on);
/* which = 0 parameters, 1 gradients (of the last pgb_net_loss_grad or
 * train step); to_device = 1 uploads (parameters only) */
int pgb_net_params(pgb_net *net, int which, float *host, int to_device);
int pgb_net_predict(pgb_net *net, const double *rho, double *u, void *stream);
/* Scales a guess u of lap u = rho (u = 0 on the boundary, uniform spacing
 * h, both device n^3 arrays) by alpha = <u, rho> / <u, lap u>, the factor
 * that minimises the error of alpha u in the energy norm of -lap: a net
 * whose shape is right but whose amplitude is off gets the amplitude from
 * the equation. Runs on the device (no host synchronisation). */
int pgb_net_rescale(pgb_net *net, const double *rho, double *u, double h, void *stream);
/* pgb_net_rescale is also the guess's guard: a guess that is not finite
 * (any NaN or Inf), is zero, or needs an amplitude factor outside
 * [1/16, 16] is replaced on the device by u = 0, the plain solve's initial
 * guess, so a corrupt prediction costs nothing but the prediction; this
 * returns how many guesses were replaced so far */
int pgb_net_rejected_guesses(pgb_net *net, long *count);
int pgb_net_loss_grad(pgb_net *net, const double *rho, const float *u_target, double *loss, void *stream);
int pgb_net_train_step(pgb_net *net, const double *rho, const float *u_target, float lr, double *loss,
                       void *stream);

#ifdef __cplusplus
}
#endif
#endif
