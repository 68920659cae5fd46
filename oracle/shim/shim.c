/*
 * Implementations behind oracle/shim/mpi.h and oracle/shim/bbhutil.h.
 *
 * TEST INFRASTRUCTURE (oracle only): links the reference's C sources into a
 * single-process CPU checker. Nothing here is used by the GPU library.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <ctype.h>
#include "mpi.h"
#include "bbhutil.h"

/* ------------------------------------------------------------------ MPI -- */
int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm c, int *rank) { (void)c; *rank = 0; return MPI_SUCCESS; }
int MPI_Comm_size(MPI_Comm c, int *size) { (void)c; *size = 1; return MPI_SUCCESS; }
int MPI_Bcast(void *b, int n, MPI_Datatype t, int r, MPI_Comm c)
{ (void)b; (void)n; (void)t; (void)r; (void)c; return MPI_SUCCESS; }

int MPI_Allreduce(void *s, void *r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c)
{
   (void)op; (void)c;
   if (s != r) memmove(r, s, (size_t)n * (size_t)t);
   return MPI_SUCCESS;
}

int MPI_Allgather(void *s, int sn, MPI_Datatype st, void *r, int rn, MPI_Datatype rt, MPI_Comm c)
{
   (void)rn; (void)rt; (void)c;
   memmove(r, s, (size_t)sn * (size_t)st);
   return MPI_SUCCESS;
}

int MPI_Allgatherv(void *s, int sn, MPI_Datatype st, void *r, int *rcounts, int *displs,
                   MPI_Datatype rt, MPI_Comm c)
{
   (void)rcounts; (void)c;
   memmove((char *)r + (size_t)displs[0] * (size_t)rt, s, (size_t)sn * (size_t)st);
   return MPI_SUCCESS;
}

static int no_peer(const char *who)
{
   fprintf(stderr, "oracle mpi shim: %s called with one rank\n", who);
   abort();
   return 1;
}
int MPI_Isend(void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c, MPI_Request *q)
{ (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; (void)q; return no_peer("MPI_Isend"); }
int MPI_Irecv(void *b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Request *q)
{ (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; (void)q; return no_peer("MPI_Irecv"); }
int MPI_Waitall(int n, MPI_Request *q, MPI_Status *st)
{ (void)q; (void)st; return n ? no_peer("MPI_Waitall") : MPI_SUCCESS; }

/* ------------------------------------------------------- parameter files -- */
/* Finds "name := value" in text; returns pointer to the value text or NULL. */
static const char *find_value(const char *text, const char *name)
{
   size_t nl = strlen(name);
   const char *line = text;
   while (line && *line) {
      const char *p = line;
      while (*p == ' ' || *p == '\t') p++;
      if (*p != '#' && strncmp(p, name, nl) == 0) {
         const char *q = p + nl;
         while (*q == ' ' || *q == '\t') q++;
         if (q[0] == ':' && q[1] == '=') {
            q += 2;
            while (*q == ' ' || *q == '\t') q++;
            return q;
         }
      }
      line = strchr(line, '\n');
      if (line) line++;
   }
   return NULL;
}

static char *slurp(const char *file)
{
   FILE *f = fopen(file, "rb");
   long n;
   char *buf;
   if (!f) return NULL;
   fseek(f, 0, SEEK_END);
   n = ftell(f);
   fseek(f, 0, SEEK_SET);
   buf = (char *)malloc((size_t)n + 1);
   if (fread(buf, 1, (size_t)n, f) != (size_t)n) { fclose(f); free(buf); return NULL; }
   buf[n] = 0;
   fclose(f);
   return buf;
}

/* numeric tokens of the value (scalar or [a b c]) */
static int parse_nums(const char *v, double *out, int size)
{
   int n = 0;
   const char *p = v;
   int bracket = 0;
   if (*p == '[') { bracket = 1; p++; }
   while (*p && *p != '\n' && n < size) {
      char *end;
      double x;
      while (*p == ' ' || *p == '\t' || *p == ',') p++;
      if (*p == ']' || *p == '\n' || !*p) break;
      x = strtod(p, &end);
      if (end == p) return -1;
      out[n++] = x;
      p = end;
      if (!bracket) break;
   }
   return n;
}

static int parse_strs(const char *v, char **out, int size)
{
   int n = 0;
   const char *p = v;
   while (*p && *p != '\n' && n < size) {
      const char *q;
      while (*p && *p != '"' && *p != '\n') p++;
      if (*p != '"') break;
      q = strchr(p + 1, '"');
      if (!q) return -1;
      out[n] = (char *)malloc((size_t)(q - p));
      memcpy(out[n], p + 1, (size_t)(q - p - 1));
      out[n][q - p - 1] = 0;
      n++;
      p = q + 1;
   }
   return n;
}

static int sget_num(char *text, char *name, double *tmp, int size)
{
   const char *v = find_value(text, name);
   int n;
   if (!v) return 0;
   n = parse_nums(v, tmp, size);
   if (n < 0) return -1;
   if (n != size) return -2;
   return 1;
}

int sget_int_param(char *string, char *name, int *var, int size)
{
   double tmp[64];
   int i, r;
   if (size > 64) return -1;
   r = sget_num(string, name, tmp, size);
   if (r == 1) for (i = 0; i < size; i++) var[i] = (int)tmp[i];
   return r;
}

int sget_real_param(char *string, char *name, double *var, int size)
{
   double tmp[256];
   int i, r;
   if (size > 256) return -1;
   r = sget_num(string, name, tmp, size);
   if (r == 1) for (i = 0; i < size; i++) var[i] = tmp[i];
   return r;
}

int sget_str_param(char *string, char *name, char **var, int size)
{
   const char *v = find_value(string, name);
   int n;
   if (!v) return 0;
   n = parse_strs(v, var, size);
   if (n < 0) return -1;
   if (n != size) return -2;
   return 1;
}

/* ivecs (output schedules) are never used by the checker: always empty */
int sget_ivec_param(char *string, char *name, int *var, int size)
{
   (void)string; (void)name; (void)size;
   var[0] = 0;
   return 1;
}

#define FILE_PARAM(kind, T)                                              \
   int get_##kind##_param(char *file, char *name, T *var, int size)     \
   {                                                                     \
      char *text = slurp(file);                                          \
      int r;                                                             \
      if (!text) return -1;                                              \
      r = sget_##kind##_param(text, name, var, size);                    \
      free(text);                                                        \
      return r;                                                          \
   }
FILE_PARAM(int, int)
FILE_PARAM(real, double)
FILE_PARAM(str, char *)

int get_ivec_param(char *file, char *name, int *var, int size)
{ (void)file; return sget_ivec_param(0, name, var, size); }

int do_ivec(int it, int niv, int *ivec) { (void)it; (void)niv; (void)ivec; return 0; }
void fixup_ivec(int min, int max, int lev, int *ivec) { (void)min; (void)max; (void)lev; (void)ivec; }

/* -------------------------------------------------------------- SDF i/o -- */
int gft_out_bbox(char *n, double t, int *s, int r, double *b, double *d)
{ (void)n; (void)t; (void)s; (void)r; (void)b; (void)d; return 1; }
int gft_out_brief(char *n, double t, int *s, int r, double *d)
{ (void)n; (void)t; (void)s; (void)r; (void)d; return 1; }
int gft_close(char *n) { (void)n; return 1; }
int gft_read_shape(char *n, int l, int *s) { (void)n; (void)l; (void)s; return 0; }
int gft_read_brief(char *n, int l, double *d) { (void)n; (void)l; (void)d; return 0; }
int gft_read_full(char *n, int l, int *s, char *c, int r, double *t, double *co, double *d)
{ (void)n; (void)l; (void)s; (void)c; (void)r; (void)t; (void)co; (void)d; return 0; }
