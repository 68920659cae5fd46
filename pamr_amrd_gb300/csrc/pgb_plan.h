/*
 * Host-side hierarchy and transfer-plan builder of libpamr_gb300 (C).
 *
 * Given the AMR grids of a PAMR hierarchy (one rank, refinement ratio 2),
 * builds the multigrid hierarchy the way PAMR_build_mgh does
 * (src/gh.c:1097-1365) and precomputes, once per hierarchy, every transfer
 * the V-cycle performs (PAMR_sync / PAMR_inject / PAMR_interp,
 * src/pamr.c:533-685 over src/transfer.c) as flat op tables, plus the two
 * cmask arrays per box (amrd/mg.c:362-488). The reference rebuilds these
 * lists on every call; here they are built once and replayed on the GPU.
 */
#ifndef PGB_PLAN_H
#define PGB_PLAN_H

#include "pgb_internal.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
   int level;            /* MG level, 1-based */
   int shape[3];
   double bbox[6];
   double *x[3];         /* coordinates as compose_cgh fills them (src/gh.c:895-899) */
   int coarsest;
   int amr_grid;         /* input grid stored by this box, -1 on pure MG levels */
   uint8_t *child_mask;  /* host copies of the cmask arrays (1 = AMRD_CMASK_ON) */
   uint8_t *bdy_mask;
   int count;            /* interior points with bdy mask ON */
   int flags;
} pgb_hbox;

typedef struct {
   int nbox;
   int *box;             /* global box indices in PAMR grid-list order */
   double dx[3];
   int in_amrh;
} pgb_hlevel;

typedef struct {
   int pre_swp, pst_swp, max_iter, min_iter, max_citer;
   double tol, crtol, w0_r, w0_i;
   int min_cwidth;
   int restr_u, restr_res, restr_src;
   int interp_order, interp_buffer;
   int precision;
   int nsrc;                          /* source fields (>= 1 allocated) */
   int restr_srck[PGB_NSRC_MAX];      /* MG restriction of each source (restr_srck[0] = restr_src) */
   int min_level;                     /* coarsest AMR level of the MG hierarchy (PAMR_build_mgh's min_lev) */
   int nvar;                          /* elliptic variables (1..PGB_NVAR_MAX) */
} pgb_hparams;

typedef struct pgb_hier {
   int dim, pde;
   int base_shape[3];
   double base_bbox[6];
   pgb_hparams prm;
   int n_amr;
   int ngrids;
   int *grid_box;          /* input grid -> box index */
   int nbox;
   pgb_hbox *boxes;
   int nlev;
   pgb_hlevel lev[PGB_MAXLEV + 1];
   /* plans, indexed by MG level */
   pgb_plan sync[PGB_MAXLEV + 1][2];     /* PAMR_sync(L,..,AMR_bdy_width=0/1) over all boxes */
   pgb_plan sync_coarsest[PGB_MAXLEV + 1];/* PAMR_sync(L,..,1) over coarsest boxes only */
   pgb_plan inject[PGB_MAXLEV + 1];      /* PAMR_inject(L+1 -> L), stored at L */
   pgb_plan inject_init[PGB_MAXLEV + 1]; /* build-time injection (TF_MGH_INIT) into L */
   pgb_plan interp[PGB_MAXLEV + 1];      /* PAMR_interp(L-1 -> L), stored at L */
   char err[256];
} pgb_hier;

/* builds the hierarchy and all plans; returns 0 or an error code */
int pgb_hier_build(pgb_hier *h, int dim, int pde, const int *base_shape, const double *base_bbox,
                   int ngrids, const int *grid_level, const double *grid_bbox,
                   const pgb_hparams *prm);
void pgb_hier_free(pgb_hier *h);

/* regrid transfers into AMR level Ln of hn from ho (init_new_cgh,
 * src/gh.c:934-1045): interpolation from ho's level Ln-1 (when interp) and
 * copies from ho's level Ln, over the joint box list ho's boxes, then hn's */
int pgb_plan_regrid(const pgb_hier *ho, const pgb_hier *hn, int Ln, int order, int interp, pgb_plan *pi,
                    pgb_plan *pc, char *err, size_t errlen);
/* PAMR_interp / PAMR_AMR_bdy_interp (src/pamr.c:623-661) from AMR level lc
 * to lc+1 as an interpolation op list of the given order (2 or 4); the
 * caller releases it with pgb_plan_release (host side) */
int pgb_plan_amr_interp(pgb_hier *h, int lc, int amr_bdy_width, int order, pgb_plan *out);
void pgb_plan_release(pgb_plan *p);

#ifdef __cplusplus
}
#endif
#endif
