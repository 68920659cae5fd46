/* Oracle restatement of AMRD's Berger-Oliger MG-variable bookkeeping
 * (amrd/evolve.c); test infrastructure only. */
#ifndef ORACLE_BO_OPS_H
#define ORACLE_BO_OPS_H

int oracle_mg_extrap(int method, double tnp1, double tnp1_lm1, double dt, double dt_lm1, double *mgf0,
                     const double *mgf1, const double *etm1, const double *etm2, long n);
void oracle_update_mg_extrap_vars(int L1, int Lf, const int *rho_tm, int ngrids, const int *level, double **etm1,
                                  double **etm2, double *const *mgf1, double *const *brs, const long *n,
                                  double eps_c);
void oracle_set_mg_brs_vars(int L1, int L2, int ngrids, const int *level, double **brs, double *const *mgf1,
                            const long *n);

#endif
