/*
 * Minimal stand-in for RNPL's libbbhutil (parameter files and SDF output).
 *
 * TEST INFRASTRUCTURE (oracle only). Parameter files use the reference's
 * "name := value" syntax (examples/nbs/nbs.fparam). SDF output is not needed
 * by the multigrid path; the gft_* entry points accept and discard data.
 */
#ifndef ORACLE_SHIM_BBHUTIL_H
#define ORACLE_SHIM_BBHUTIL_H

int get_int_param(char *file, char *name, int *var, int size);
int get_real_param(char *file, char *name, double *var, int size);
int get_str_param(char *file, char *name, char **var, int size);
int get_ivec_param(char *file, char *name, int *var, int size);
int sget_int_param(char *string, char *name, int *var, int size);
int sget_real_param(char *string, char *name, double *var, int size);
int sget_str_param(char *string, char *name, char **var, int size);
int sget_ivec_param(char *string, char *name, int *var, int size);
int do_ivec(int it, int niv, int *ivec);
void fixup_ivec(int min, int max, int lev, int *ivec);

int gft_out_bbox(char *name, double time, int *shape, int rank, double *bbox, double *data);
int gft_out_brief(char *name, double time, int *shape, int rank, double *data);
int gft_close(char *name);
int gft_read_shape(char *name, int level, int *shape);
int gft_read_brief(char *name, int level, double *data);
int gft_read_full(char *name, int level, int *shape, char *cnames, int rank, double *time,
                  double *coords, double *data);

#endif
