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
enum { ORACLE_POISSON = 0, ORACLE_CONFORMAL = 1, ORACLE_LAPSE = 2, ORACLE_NBS = 3 };

/* number of source grid functions a PDE kind reads */
int oracle_nsrc(int pde);

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

#endif
