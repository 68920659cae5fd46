/*
 * Internal structures shared by the C host code (hierarchy/plan builder,
 * V-cycle driver) and the CUDA kernels of libpamr_gb300.
 *
 * Terminology follows PAMR/AMRD: an AMR "grid" becomes an MG "box" on every
 * MG level; grid functions per box are u (the elliptic variable f), res
 * (f_res), lop (f_lop), rhs (f_rhs) and src (the source variable the
 * operator reads); cmask is kept as two byte masks per box (child mask for
 * L_op/compute_MG_rhs, boundary mask for relax/residual).
 */
#ifndef PGB_INTERNAL_H
#define PGB_INTERNAL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* grid functions, in PAMR gfn order for the AMRD variable set
 * (hyperbolic source first, then f, f_res, f_lop, f_rhs; amrd/io.c:708-937);
 * sources 1..3 of an operator with several source fields follow (their
 * arrays exist only when the operator reads them) */
enum { PGB_F_SRC = 0, PGB_F_U = 1, PGB_F_RES = 2, PGB_F_LOP = 3, PGB_F_RHS = 4, PGB_F_SRC1 = 5,
       PGB_F_VAR1 = 8, PGB_NF = 20 };
#define PGB_NSRC_MAX 4
#define PGB_SRC_FIELD(k) ((k) ? PGB_F_SRC1 + (k) - 1 : PGB_F_SRC)
/* Elliptic variables (AMRD_num_elliptic_vars, amrd/mg.c:248): variable 0
 * uses PGB_F_U..PGB_F_RHS, variable v > 0 the four fields from
 * PGB_F_VAR1 + 4 (v - 1) in the same order (their arrays exist only for the
 * solver's variables). PGB_FV(v, f) maps f in {U, RES, LOP, RHS}. */
#define PGB_NVAR_MAX 4
#define PGB_FV(v, f) ((v) ? PGB_F_VAR1 + 4 * ((v) - 1) + ((f) - PGB_F_U) : (f))
/* field mask of f over variables 0..n-1 */
#define PGB_VMASK(n, f) pgb_vmask((n), (f))
static inline int pgb_vmask(int n, int f)
{
   int m = 0, v;
   for (v = 0; v < n; v++) m |= 1 << PGB_FV(v, f);
   return m;
}
/* field mask of sources 0..n-1 */
#define PGB_SRC_MASK(n) ((1 << PGB_F_SRC) | ((((1 << ((n) > 1 ? (n) - 1 : 0)) - 1)) << PGB_F_SRC1))

/* Device form of a level operator L[u] = (program of lap u, u, sources)
 * and its diagonal dL/du: a short stack program of one-byte instructions
 * (low 4 bits opcode, high 4 bits argument: source or constant index),
 * evaluated left to right in IEEE double arithmetic, one rounding per
 * operation, so that an operator written in the order of an application's
 * hook (e.g. examples/nbs/num.f:113-116) rounds exactly like it. kind
 * selects a compiled form for the built-in operators (same arithmetic). */
#define PGB_PROG_MAX 32
#define PGB_PROG_CONST 8
#define PGB_PROG_STACK 8
/* PGB_P_U's argument: 0 = the variable the equation belongs to, 1 + k =
 * variable k (expression names u0..u3) */
enum { PGB_P_END = 0, PGB_P_LAP, PGB_P_J0, PGB_P_U, PGB_P_SRC, PGB_P_CONST, PGB_P_ADD, PGB_P_SUB,
       PGB_P_MUL, PGB_P_DIV, PGB_P_NEG };
enum { PGB_OPK_POISSON = 0, PGB_OPK_CONFORMAL = 1, PGB_OPK_LAPSE = 2, PGB_OPK_PROGRAM = 3 };
typedef struct {
   int kind;                            /* PGB_OPK_* */
   int nsrc;                            /* source fields the operator reads (0..PGB_NSRC_MAX) */
   unsigned char lcode[PGB_PROG_MAX];   /* L[u] */
   unsigned char jcode[PGB_PROG_MAX];   /* dL/du */
   double cst[PGB_PROG_CONST];
   int nvread;   /* one-variable kernels (mixed form) running variable v of several: the
                  * variables 0..nvread-1 the program names are read from the box's
                  * variable fields at the point (0: the program names only u) */
   int cfixed;   /* mixed form, several variables: no coupling coefficient dL/du_k depends
                  * on lap or a variable (pgb_dop_couplings_fixed), so they are computed
                  * once per pgb_prepare */
   int jfixed;   /* the same for the Jacobian term dL/du - j0 (pgb_dop_jac_fixed) */
} pgb_dop;
int pgb_dop_couplings_fixed(const pgb_dop *d);
int pgb_dop_jac_fixed(const pgb_dop *d);

#define PGB_MAXLEV 48

/* box flags */
#define PGB_BOX_POW2DX 1     /* every dx^2 is a power of two: x/dx2 == x*(1/dx2) exactly */
#define PGB_BOX_BDY_INTERIOR 2 /* the boundary cmask is ON at every interior point */
#define PGB_BOX_COARSEST 4
#define PGB_BOX_ISO 8         /* dx^2 is the same in every dimension */

/* device view of one MG box (all pointers are device pointers) */
#define PGB_NW32 5   /* FP32 work arrays per box (mixed form) */
#define PGB_W32_E 0   /* slot of the correction E a smoothing block starts from */
#define PGB_W32_D 1   /* FP32 defect D (-res after the residual pass) */
#define PGB_W32_E2 4  /* second correction slot of the fused sweeps */

typedef struct {
   double *f[PGB_NF];
   const pgb_dop *op;            /* the level operator (device copy) */
   const uint8_t *cmask_child;   /* set_cmask_child, amrd/mg.c:362-426 */
   const uint8_t *cmask_bdy;     /* set_cmask_bdy, amrd/mg.c:432-488 */
   float *w32[PGB_NW32];         /* mixed form: correction, defect, Jacobian term, coarse correction,
                                  * second correction buffer (fused sweeps write it) */
   float *w32c;                  /* mixed form, several variables: dL/du_k of the box's variable for the
                                  * variables in slots k = 1..nvar-1, one FP32 array each (same layout
                                  * and pitch as w32, wz * Nz floats apart); 0 with one variable */
   int n[3];                     /* Nx, Ny, Nz (Nz = 1 in 2-D) */
   int wy;                       /* FP32 arrays: row pitch (Nx rounded up to 4 floats, so every row
                                  * starts on 16 bytes: vector and TMA loads) */
   long wz;                      /* FP32 arrays: plane pitch wy * Ny */
   int flags;
   int level;
   int count;                    /* # interior points with cmask_bdy ON (norm divisor) */
   double dx2[3];                /* (x(2)-x(1))^2 per dimension */
   double idx2[3];               /* 1/dx2 when PGB_BOX_POW2DX */
   double j0;                    /* -2/dx2 - 2/dy2 [- 2/dz2] */
   float fidx2[3], fj0;          /* FP32 copies of idx2 and j0 (mixed form) */
} pgb_dbox;

/* a tile of a box processed by one CTA */
typedef struct {
   int box;          /* global box index */
   int i0, j0, k0;   /* 0-based tile origin */
   int slot;         /* partial-sum slot of the box-local reduction */
} pgb_tile;

/* restriction (inject) op: src/transfer.c:1126-1149 + m_util_r8.f:20-50,649-830 */
typedef struct {
   int src_box, dst_box;
   int i1, j1, k1;        /* fine start, 1-based */
   int i2, j2, k2;        /* coarse start, 1-based */
   int ni, nj, nk;        /* coarse extents */
   int irho;
   int op[PGB_NF];        /* per grid function: 0 none, 1 straight, 2 HW, 3 FW */
} pgb_restrict_op;

/* in-level copy (sync): src/transfer.c:1074-1079 */
typedef struct {
   int src_box, dst_box;
   int i1, j1, k1, i2, j2, k2, ni, nj, nk;
} pgb_copy_op;

/* coarse -> fine interpolation: src/transfer.c:1007-1116 + dminterp3d */
typedef struct {
   int src_box, dst_box;
   int i1i, j1i, k1i;     /* coarse window start, 1-based */
   int nii, nji, nki;     /* window anchors per dimension */
   int i2b, j2b, k2b;     /* start inside the interpolated window, 1-based */
   int i2, j2, k2;        /* fine start, 1-based */
   int nib, njb, nkb;     /* fine extents */
   int irho, ord;
} pgb_interp_op;

/* a list of ops executed as ordered batches; ops within a batch write
 * disjoint points */
typedef struct {
   int nops;
   int nbatch;
   int *batch_start;       /* host, nbatch+1 */
   int *batch_maxpts;      /* host, largest op (in points) of each batch */
   void *h_ops;            /* host copy */
   void *d_ops;            /* device copy */
} pgb_plan;

#ifdef __cplusplus
}
#endif
#endif
