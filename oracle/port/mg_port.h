/*
 * Oracle port: a plain-C restatement of the reference's multigrid path
 * (amrd/mg.c over PAMR's MG hierarchy, src/gh.c + src/transfer.c +
 * src/pamr.c, one rank) for use as the CPU checker and the timed CPU
 * baseline on machines where the reference itself is not built.
 *
 * TEST INFRASTRUCTURE: only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline arm use it. It is pinned against the compiled reference
 * (oracle/_ref) by tests/test_oracle_port.py.
 *
 * Scope: refinement ratio 2 between AMR levels, no excision, no periodic
 * boundaries, single rank (the configuration the GPU library reproduces).
 */
#ifndef ORACLE_MG_PORT_H
#define ORACLE_MG_PORT_H

typedef struct {
   int dim, pde, ngrids;
   int base_shape[3];
   double base_bbox[6];
   const int *lev;         /* AMR level of each input grid (1-based) */
   const double *bbox;     /* 6 doubles per input grid */
   double **u;             /* in: initial guess, out: solution (per input grid) */
   const double *const *src;
   int pre_swp, pst_swp, max_iter, min_iter, max_citer;
   double tol, crtol, w0_r, w0_i;
   int min_cwidth;
   int restr_u, restr_res, restr_src;  /* 1 straight, 2 half weight, 3 full weight */
   int interp_order;                   /* 2 or 4 */
   int interp_buffer;                  /* PAMR default 2 (src/pamr.c:157) */
   /* sources beyond the first (oracle_nsrc(pde) - 1 of them): srcx[k][i] is
    * source k+1 of input grid i, restricted with restr_srcx[k] */
   const double *const *srcx[3];
   int restr_srcx[3];
   int min_level;                      /* coarsest AMR level of the MG hierarchy (solve_elliptics' L) */
} port_case;

typedef struct {
   int iters;
   int n_levels;
   double *res;           /* per V-cycle finest residual, capacity max_iter */
   /* optional hook log (relax=0, residual=1, lop=2): capacity hk_cap */
   int hk_cap, hk_n;
   int *hk_kind, *hk_L, *hk_idx;
   double *hk_norm;
} port_result;

/* returns 0 on success, nonzero on invalid input */
int port_solve(const port_case *c, port_result *r);

#endif
