/*
 * Prototypes of the C restatement of src/m_util_r8.f (oracle/m_util_r8.c).
 * TEST INFRASTRUCTURE (oracle only). Signatures follow include/m_util_r8.h:
 * Fortran calling convention, every argument by pointer, trailing underscore.
 */
#ifndef ORACLE_M_UTIL_R8_C_H
#define ORACLE_M_UTIL_R8_C_H

void dmcopy3d_(double *u1, double *u2, int *nx1, int *ny1, int *nz1, int *nx2, int *ny2, int *nz2,
               int *i1, int *j1, int *k1, int *i2, int *j2, int *k2, int *ni, int *nj, int *nk,
               int *si1, int *sj1, int *sk1, int *si2, int *sj2, int *sk2);
void dminterp3d_(double *u1, double *u2, int *nx1, int *ny1, int *nz1, int *nx2, int *ny2,
                 int *nz2, int *i1, int *j1, int *k1, int *i2, int *j2, int *k2, int *ni, int *nj,
                 int *nk, int *si1, int *sj1, int *sk1, int *irho, int *jrho, int *krho, int *ord,
                 double *chr1, double *ex, int *do_ex);
void dmhwr3d_(double *u1, double *u2, int *nx1, int *ny1, int *nz1, int *nx2, int *ny2, int *nz2,
              int *i1, int *j1, int *k1, int *i2, int *j2, int *k2, int *ni, int *nj, int *nk,
              int *si1, int *sj1, int *sk1, int *si2, int *sj2, int *sk2, double *chr1,
              double *ex, int *do_ex);
void dmfwr3d_(double *u1, double *u2, int *nx1, int *ny1, int *nz1, int *nx2, int *ny2, int *nz2,
              int *i1, int *j1, int *k1, int *i2, int *j2, int *k2, int *ni, int *nj, int *nk,
              int *si1, int *sj1, int *sk1, int *si2, int *sj2, int *sk2, double *chr1,
              double *ex, int *do_ex);

/* call log (see oracle/m_util_r8.c) */
enum { MUR8_COPY = 1, MUR8_INTERP = 2, MUR8_HWR = 3, MUR8_FWR = 4 };
#define MUR8_NARGS 24
typedef struct {
   int kind;
   const double *u1, *u2;
   int iv[MUR8_NARGS];
} mur8_call;
extern int mur8_log_enabled;
extern mur8_call *mur8_log;
extern int mur8_log_n, mur8_log_cap;

#endif
