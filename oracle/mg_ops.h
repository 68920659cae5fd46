/*
 * Per-grid elliptic operators for the CPU checker, written in the pattern of
 * the reference application hooks examples/nbs/num.f:85-246 (lop, residual,
 * relax) and w/examples/nps/num_w.f:18-158 (Poisson form).
 *
 * TEST INFRASTRUCTURE (oracle only). The GPU library implements the same
 * operators with the same expression order; these are the checker's copy.
 */
#ifndef ORACLE_MG_OPS_H
#define ORACLE_MG_OPS_H

/* PDE kinds: L[u] = lap(u) + term(src,u)
 *   ORACLE_POISSON   : term = -src                  (lap u = rho)
 *   ORACLE_CONFORMAL : term = +2*pi*src*u^5         (Hamiltonian constraint, psi)
 *   ORACLE_LAPSE     : term = -src*u                (maximal-slicing lapse)
 *   ORACLE_NBS       : term = -(src0^2 + src1^2)    (the Newtonian boson star's
 *                      potential V_xx+V_yy+V_zz - (phi_r^2+phi_i^2),
 *                      examples/nbs/num.f:113-116; two sources) */
enum { ORACLE_POISSON = 0, ORACLE_CONFORMAL = 1, ORACLE_LAPSE = 2, ORACLE_NBS = 3, ORACLE_COUPLED = 4 };

/* number of source grid functions a PDE kind reads */
int oracle_nsrc(int pde);
/* number of elliptic variables: 2 for ORACLE_COUPLED (u, w), else 1 */
int oracle_nvar(int pde);

#define ORACLE_CMASK_ON 1.0

typedef struct {
   int dim;
   int shape[3];  /* Nx,Ny,Nz (Nz=1 in 2-D) */
   double dx[3];  /* x(2)-x(1) of the grid's coordinate arrays */
} oracle_grid;

/* src: oracle_nsrc(pde) source arrays */
void oracle_lop(int pde, const oracle_grid *g, double *lv, const double *v, const double *const *src,
                const double *cmask);
double oracle_residual(int pde, const oracle_grid *g, double *res, const double *rhs,
                       const double *v, const double *const *src, const double *cmask);
double oracle_relax(int pde, const oracle_grid *g, double *v, const double *rhs,
                    const double *const *src, const double *cmask);

/* ORACLE_COUPLED, two elliptic variables (u, w) handled together by each
 * hook, as an application with several elliptic variables writes them:
 *   L_u = lap u - s0*(u - w) - s1,   dL_u/du = j0 - s0
 *   L_w = lap w - s0*(w - u),        dL_w/dw = j0 - s0
 * relax updates u, then w, at each point of a colour (w from the new u);
 * the norms sum both variables' squared residuals over the points.
 * v, lv, res, rhs: one array per variable. */
void oracle_lop_n(int pde, const oracle_grid *g, double *const *lv, const double *const *v,
                  const double *const *src, const double *cmask);
double oracle_residual_n(int pde, const oracle_grid *g, double *const *res, const double *const *rhs,
                         const double *const *v, const double *const *src, const double *cmask);
double oracle_relax_n(int pde, const oracle_grid *g, double *const *v, const double *const *rhs,
                      const double *const *src, const double *cmask);

#endif
