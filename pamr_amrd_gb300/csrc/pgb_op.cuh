/*
 * Device evaluation of a level operator (pgb_dop, pgb_internal.h): the
 * program of L[u] and of dL/du at one point, every operation rounded once
 * in IEEE double (explicit _rn intrinsics, so no FMA contraction whatever
 * the translation unit's -fmad setting). Shared by the FP64 kernels and the
 * FP64 passes of the mixed form.
 */
#ifndef PGB_OP_CUH
#define PGB_OP_CUH

#include "pgb_internal.h"

/* the source values an operator reads at point p of box b; s0 is passed
 * in (some kernels hold it in shared memory), the others come from the
 * box's source arrays */
struct pgb_srcv {
   double s0, s1, s2, s3;
};

static __device__ __forceinline__ pgb_srcv pgb_load_src(int nsrc, const pgb_dbox &b, long p, double s0)
{
   pgb_srcv v;
   v.s0 = s0;
   v.s1 = nsrc > 1 ? b.f[PGB_F_SRC1][p] : 0.0;
   v.s2 = nsrc > 2 ? b.f[PGB_F_SRC1 + 1][p] : 0.0;
   v.s3 = nsrc > 3 ? b.f[PGB_F_SRC1 + 2][p] : 0.0;
   return v;
}

/* runs one program; lapv/j0 are the values of the names lap and j0, u
 * the equation's own variable, uv[k] variable k (the names u0..u3; uv = 0
 * with one variable, where u0 is u) */
static __device__ __noinline__ double pgb_prog_run(const unsigned char *code, const double *cst, double lapv, double j0,
                                            double u, const double *uv, pgb_srcv s)
{
   double st[PGB_PROG_STACK];
   double top = 0.0;
   int sp = 0;
   for (int q = 0; q < PGB_PROG_MAX; q++) {
      const unsigned c = code[q];
      const unsigned opc = c & 15u, arg = c >> 4;
      double v;
      if (opc == PGB_P_END) break;
      switch (opc) {
      case PGB_P_LAP: v = lapv; break;
      case PGB_P_J0: v = j0; break;
      case PGB_P_U: v = arg && uv ? uv[arg - 1] : u; break;
      case PGB_P_SRC: v = arg == 0 ? s.s0 : arg == 1 ? s.s1 : arg == 2 ? s.s2 : s.s3; break;
      case PGB_P_CONST: v = cst[arg]; break;
      case PGB_P_NEG: top = -top; continue;
      default: {
         const double a = st[--sp];
         if (opc == PGB_P_ADD) top = __dadd_rn(a, top);
         else if (opc == PGB_P_SUB) top = __dsub_rn(a, top);
         else if (opc == PGB_P_MUL) top = __dmul_rn(a, top);
         else top = __ddiv_rn(a, top);
         continue;
      }
      }
      if (q > 0) st[sp++] = top;   /* push the old top (nothing lies below the first value) */
      top = v;
   }
   return top;
}

/* A program of one variable of several run by a one-variable kernel (the
 * mixed form's passes over a variable's view of the boxes, where the
 * variable's own fields sit in the slots of variable 0 and the program's
 * names are renumbered to match): uv[0] = u, uv[k] is read from the box's
 * field of variable k at the point (uk = that field + p). Kept out of line
 * so that the one-variable call sites keep their registers. */
static __device__ __noinline__ double pgb_prog_run_vars(const unsigned char *code, const double *cst, double lapv,
                                                        double j0, double u, int nvread, const double *u1,
                                                        const double *u2, const double *u3, pgb_srcv s)
{
   double uv[PGB_NVAR_MAX];
   uv[0] = u;
   uv[1] = *u1;
   uv[2] = nvread > 2 ? *u2 : 0.0;
   uv[3] = nvread > 3 ? *u3 : 0.0;
   return pgb_prog_run(code, cst, lapv, j0, u, uv, s);
}

static __device__ __forceinline__ double pgb_prog_any(const pgb_dbox &b, const unsigned char *code, double lapv,
                                                      double u, double s0, long p)
{
   const pgb_dop *o = b.op;
   const pgb_srcv sv = pgb_load_src(o->nsrc, b, p, s0);
   if (o->nvread < 2) return pgb_prog_run(code, o->cst, lapv, b.j0, u, 0, sv);
   const int nr = o->nvread;
   return pgb_prog_run_vars(code, o->cst, lapv, b.j0, u, nr, b.f[PGB_FV(1, PGB_F_U)] + p,
                            nr > 2 ? b.f[PGB_FV(2, PGB_F_U)] + p : 0, nr > 3 ? b.f[PGB_FV(3, PGB_F_U)] + p : 0, sv);
}

/* The derivative of a program's value with respect to the variable in
 * slot ws >= 1 of uv (forward-mode differentiation: every value carries its
 * derivative through the same operations; lap, j0, u, the sources and the
 * constants do not depend on it). Plain double arithmetic: the mixed form's
 * coupled FP32 smoother takes it as its coupling coefficient. */
static __device__ __noinline__ double pgb_prog_dvar(const unsigned char *code, const double *cst, double lapv,
                                                    double j0, double u, const double *uv, pgb_srcv s, int ws)
{
   double st[PGB_PROG_STACK], ds[PGB_PROG_STACK];
   double top = 0.0, dtop = 0.0;
   int sp = 0;
   for (int q = 0; q < PGB_PROG_MAX; q++) {
      const unsigned c = code[q];
      const unsigned opc = c & 15u, arg = c >> 4;
      double v, dv = 0.0;
      if (opc == PGB_P_END) break;
      switch (opc) {
      case PGB_P_LAP: v = lapv; break;
      case PGB_P_J0: v = j0; break;
      case PGB_P_U:
         v = arg ? uv[arg - 1] : u;
         dv = (int)arg == ws + 1 ? 1.0 : 0.0;
         break;
      case PGB_P_SRC: v = arg == 0 ? s.s0 : arg == 1 ? s.s1 : arg == 2 ? s.s2 : s.s3; break;
      case PGB_P_CONST: v = cst[arg]; break;
      case PGB_P_NEG:
         top = -top;
         dtop = -dtop;
         continue;
      default: {
         --sp;
         const double a = st[sp], da = ds[sp];
         if (opc == PGB_P_ADD) dtop = da + dtop, top = a + top;
         else if (opc == PGB_P_SUB) dtop = da - dtop, top = a - top;
         else if (opc == PGB_P_MUL) dtop = da * top + a * dtop, top = a * top;
         else dtop = (da * top - a * dtop) / (top * top), top = a / top;
         continue;
      }
      }
      if (q > 0) {
         st[sp] = top;
         ds[sp] = dtop;
         sp++;
      }
      top = v;
      dtop = dv;
   }
   return dtop;
}

/* L[u] and dL/du of a program operator at point p of box b (the box
 * carries a device pointer to its level operator) */
static __device__ __forceinline__ double pgb_prog_L(const pgb_dbox &b, double lapv, double u, double s0, long p)
{
   const pgb_dop *o = b.op;
   return pgb_prog_run(o->lcode, o->cst, lapv, b.j0, u, 0, pgb_load_src(o->nsrc, b, p, s0));
}

static __device__ __forceinline__ double pgb_prog_J(const pgb_dbox &b, double u, double s0, long p)
{
   const pgb_dop *o = b.op;
   return pgb_prog_run(o->jcode, o->cst, 0.0, b.j0, u, 0, pgb_load_src(o->nsrc, b, p, s0));
}

/* the same where the box table may be a variable's view (the mixed form's
 * one-variable passes): the other variables the program names are read at p */
static __device__ __forceinline__ double pgb_prog_Lview(const pgb_dbox &b, double lapv, double u, double s0, long p)
{
   return pgb_prog_any(b, b.op->lcode, lapv, u, s0, p);
}

static __device__ __forceinline__ double pgb_prog_Jview(const pgb_dbox &b, double u, double s0, long p)
{
   return pgb_prog_any(b, b.op->jcode, 0.0, u, s0, p);
}

/* the same for variable v of a solver with several elliptic variables: its
 * operator is b.op[v], uv[k] holds variable k at the point */
static __device__ __forceinline__ double pgb_prog_Lv(const pgb_dbox &b, int v, double lapv, const double *uv,
                                                     pgb_srcv s)
{
   const pgb_dop *o = b.op + v;
   return pgb_prog_run(o->lcode, o->cst, lapv, b.j0, uv[v], uv, s);
}

static __device__ __forceinline__ double pgb_prog_Jv(const pgb_dbox &b, int v, const double *uv, pgb_srcv s)
{
   const pgb_dop *o = b.op + v;
   return pgb_prog_run(o->jcode, o->cst, 0.0, b.j0, uv[v], uv, s);
}

#endif
