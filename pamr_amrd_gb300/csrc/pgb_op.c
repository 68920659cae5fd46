/*
 * Level operators of libpamr_gb300: compiles an application's elliptic
 * operator, written as two arithmetic expressions, into the device program
 * the kernels evaluate (pgb_dop in pgb_internal.h).
 *
 * In AMRD the operator lives in the application's hooks app_L_op,
 * app_MG_residual and app_MG_relax (include/amrd.h:137-159), host functions
 * over raw grid pointers (examples/nbs/num.f:85-246). A GPU solve needs the
 * same arithmetic on the device, so the application states it once:
 *
 *    L[u]  = expression of lap, u, s0..s3 and numeric constants
 *    dL/du = expression of j0, u, s0..s3 and numeric constants
 *
 * (with several elliptic variables, one such pair per variable: u is the
 * equation's own variable and u0..u3 name variable k at the same point, as
 * an application's hooks couple their variables point by point)
 *
 * where lap is the 5/7-point Laplacian of u as the hook pattern forms it
 * (num.f:113-115), j0 its diagonal -2/dx^2 - 2/dy^2 [- 2/dz^2] (num.f:236),
 * and sK the K-th source grid function at the point. Operators of equal
 * precedence associate to the left, as in Fortran and C, and every
 * operation rounds once in IEEE double, so an expression written in the
 * order of the hook reproduces the hook's results bit for bit: the nbs
 * operator V_xx+V_yy+V_zz - (phi_r^2+phi_i^2) is "lap - (s0*s0 + s1*s1)".
 * Relaxation is u <- u - (L[u] - rhs) / (dL/du) at each point, as in
 * num.f:226-238.
 */
#include <ctype.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "pamr_gb300.h"
#include "pgb_internal.h"

struct pgb_operator {
   pgb_dop d;
   char lexpr[256], jexpr[256];
};

void pgb_note_error(const char *msg);

/* the built-in operators, in the order of their hooks (oracle pattern of
 * examples/nbs/num.f:85-246): Poisson lap u = rho; conformal factor
 * lap psi + 2 pi rho psi^5 = 0 with the Newton diagonal j0 + 10 pi rho psi^4;
 * maximal-slicing lapse lap alpha = alpha S */
static const char *const BUILTIN_L[3] = {
   "lap - s0",
   "lap + 6.283185307179586*s0*(((u*u)*(u*u))*u)",
   "lap - s0*u"};
static const char *const BUILTIN_J[3] = {
   "j0",
   "j0 + 31.41592653589793*s0*((u*u)*(u*u))",
   "j0 - s0"};

typedef struct {
   const char *p;
   unsigned char *code;
   int n, depth, maxdepth;
   double *cst;
   int *ncst;
   int nsrc;
   int allow_lap;     /* lap in L, j0 in dL/du */
   char err[160];
} cparse;

static void perr(cparse *c, const char *msg)
{
   if (!c->err[0]) snprintf(c->err, sizeof(c->err), "%s at \"%.24s\"", msg, c->p);
}

static void skip(cparse *c)
{
   while (*c->p && isspace((unsigned char)*c->p)) c->p++;
}

static void emit(cparse *c, int opc, int arg, int push)
{
   if (c->n >= PGB_PROG_MAX - 1) {
      perr(c, "expression too long");
      return;
   }
   c->code[c->n++] = (unsigned char)(opc | (arg << 4));
   c->depth += push;
   if (c->depth > c->maxdepth) c->maxdepth = c->depth;
}

static int const_index(cparse *c, double v)
{
   int k;
   for (k = 0; k < *c->ncst; k++)
      if (memcmp(&c->cst[k], &v, sizeof(v)) == 0) return k;
   if (*c->ncst >= PGB_PROG_CONST) {
      perr(c, "too many distinct constants");
      return 0;
   }
   c->cst[*c->ncst] = v;
   return (*c->ncst)++;
}

static void expr(cparse *c);

static void primary(cparse *c, int neg)
{
   skip(c);
   if (c->err[0]) return;
   if (*c->p == '(') {
      c->p++;
      expr(c);
      skip(c);
      if (*c->p != ')') {
         perr(c, "missing )");
         return;
      }
      c->p++;
      if (neg) emit(c, PGB_P_NEG, 0, 0);
      return;
   }
   if (isdigit((unsigned char)*c->p) || *c->p == '.') {
      char *end;
      double v = strtod(c->p, &end);   /* correctly rounded, like a compiler's literal */
      if (end == c->p) {
         perr(c, "bad number");
         return;
      }
      c->p = end;
      emit(c, PGB_P_CONST, const_index(c, neg ? -v : v), 1);
      return;
   }
   if (isalpha((unsigned char)*c->p)) {
      char id[16];
      int n = 0;
      while (isalnum((unsigned char)*c->p) && n < 15) id[n++] = *c->p++;
      id[n] = 0;
      if (!strcmp(id, "lap") && c->allow_lap) emit(c, PGB_P_LAP, 0, 1);
      else if (!strcmp(id, "j0") && !c->allow_lap) emit(c, PGB_P_J0, 0, 1);
      else if (!strcmp(id, "u")) emit(c, PGB_P_U, 0, 1);
      else if (id[0] == 'u' && isdigit((unsigned char)id[1]) && !id[2] && id[1] - '0' < PGB_NVAR_MAX)
         emit(c, PGB_P_U, 1 + (id[1] - '0'), 1);
      else if (id[0] == 's' && isdigit((unsigned char)id[1]) && !id[2] && id[1] - '0' < c->nsrc)
         emit(c, PGB_P_SRC, id[1] - '0', 1);
      else {
         perr(c, "unknown name (lap in L, j0 in dL/du, u, u0..u3, s0.. below the source count)");
         return;
      }
      if (neg) emit(c, PGB_P_NEG, 0, 0);
      return;
   }
   perr(c, "expected a number, a name or (");
}

static void unary(cparse *c)
{
   skip(c);
   if (*c->p == '-') {
      c->p++;
      skip(c);
      /* -number folds into the constant (exact); -x negates (exact) */
      primary(c, 1);
      return;
   }
   if (*c->p == '+') c->p++;
   primary(c, 0);
}

static void term(cparse *c)
{
   unary(c);
   for (;;) {
      skip(c);
      if (c->err[0]) return;
      if (*c->p == '*' || *c->p == '/') {
         int op = *c->p == '*' ? PGB_P_MUL : PGB_P_DIV;
         c->p++;
         unary(c);
         emit(c, op, 0, -1);
      } else
         return;
   }
}

static void expr(cparse *c)
{
   term(c);
   for (;;) {
      skip(c);
      if (c->err[0]) return;
      if (*c->p == '+' || *c->p == '-') {
         int op = *c->p == '+' ? PGB_P_ADD : PGB_P_SUB;
         c->p++;
         term(c);
         emit(c, op, 0, -1);
      } else
         return;
   }
}

static int compile(const char *src, int nsrc, int is_l, unsigned char *code, double *cst, int *ncst,
                   char *err, size_t errsz)
{
   cparse c;
   memset(&c, 0, sizeof(c));
   c.p = src;
   c.code = code;
   c.cst = cst;
   c.ncst = ncst;
   c.nsrc = nsrc;
   c.allow_lap = is_l;
   memset(code, 0, PGB_PROG_MAX);
   expr(&c);
   skip(&c);
   if (!c.err[0] && *c.p) perr(&c, "unexpected text");
   if (!c.err[0] && c.maxdepth > PGB_PROG_STACK) perr(&c, "expression nests too deeply");
   if (!c.err[0] && c.depth != 1) perr(&c, "malformed expression");
   if (c.err[0]) {
      snprintf(err, errsz, "%s: %s", is_l ? "L[u]" : "dL/du", c.err);
      return 1;
   }
   code[c.n] = PGB_P_END;
   return 0;
}

static int op_build(int nsrc, const char *lexpr, const char *jexpr, pgb_operator *op, char *err,
                    size_t errsz)
{
   int ncst = 0, k;
   memset(op, 0, sizeof(*op));
   if (!lexpr || !jexpr) {
      snprintf(err, errsz, "both expressions are required");
      return 1;
   }
   if (nsrc < 0 || nsrc > PGB_NSRC_MAX) {
      snprintf(err, errsz, "source count %d out of range 0..%d", nsrc, PGB_NSRC_MAX);
      return 1;
   }
   if (strlen(lexpr) >= sizeof(op->lexpr) || strlen(jexpr) >= sizeof(op->jexpr)) {
      snprintf(err, errsz, "expression longer than %d characters", (int)sizeof(op->lexpr) - 1);
      return 1;
   }
   op->d.nsrc = nsrc;
   if (compile(lexpr, nsrc, 1, op->d.lcode, op->d.cst, &ncst, err, errsz) ||
       compile(jexpr, nsrc, 0, op->d.jcode, op->d.cst, &ncst, err, errsz))
      return 1;
   strcpy(op->lexpr, lexpr);
   strcpy(op->jexpr, jexpr);
   op->d.kind = PGB_OPK_PROGRAM;
   /* the compiled form of a built-in operator when the program is one */
   for (k = 0; k < 3 && nsrc == 1; k++) {
      pgb_operator b;
      int nb = 0;
      char e2[8];
      memset(&b, 0, sizeof(b));
      if (compile(BUILTIN_L[k], 1, 1, b.d.lcode, b.d.cst, &nb, e2, sizeof(e2)) ||
          compile(BUILTIN_J[k], 1, 0, b.d.jcode, b.d.cst, &nb, e2, sizeof(e2)))
         continue;
      if (!memcmp(b.d.lcode, op->d.lcode, PGB_PROG_MAX) && !memcmp(b.d.jcode, op->d.jcode, PGB_PROG_MAX) &&
          !memcmp(b.d.cst, op->d.cst, sizeof(b.d.cst)))
         op->d.kind = k;
   }
   /* PGB_OP_INTERPRET=1 evaluates every operator through its program (the
    * built-in compiled forms round identically; tests compare the two) */
   {
      const char *e = getenv("PGB_OP_INTERPRET");
      if (e && !strcmp(e, "1")) op->d.kind = PGB_OPK_PROGRAM;
   }
   return 0;
}

int pgb_operator_create(int nsrc, const char *lexpr, const char *jexpr, pgb_operator **out)
{
   char err[224];
   pgb_operator *op = (pgb_operator *)calloc(1, sizeof(*op));
   *out = 0;
   if (!op) {
      pgb_note_error("out of memory");
      return 1;
   }
   if (op_build(nsrc, lexpr, jexpr, op, err, sizeof(err))) {
      free(op);
      pgb_note_error(err);
      return 1;
   }
   *out = op;
   return 0;
}

int pgb_operator_builtin(int pde, pgb_operator **out)
{
   *out = 0;
   if (pde < 0 || pde > 2) {
      char m[64];
      snprintf(m, sizeof(m), "unknown pde kind %d", pde);
      pgb_note_error(m);
      return 1;
   }
   return pgb_operator_create(1, BUILTIN_L[pde], BUILTIN_J[pde], out);
}

void pgb_operator_destroy(pgb_operator *op) { free(op); }

int pgb_operator_nsrc(const pgb_operator *op) { return op ? op->d.nsrc : -1; }

int pgb_operator_kind(const pgb_operator *op) { return op ? op->d.kind : -1; }

/* the device form (library internal) */
const pgb_dop *pgb_operator_device_form(const pgb_operator *op) { return &op->d; }

/* Host evaluation of a program at one point, with the same single rounding
 * per operation as the device. */
static double prog_eval_host(const unsigned char *code, const double *cst, double lapv, double j0, double u,
                             const double *uv, const double *s)
{
   double st[PGB_PROG_STACK + 1];
   int sp = 0, q;
   for (q = 0; q < PGB_PROG_MAX && (code[q] & 15) != PGB_P_END; q++) {
      const int opc = code[q] & 15, arg = code[q] >> 4;
      switch (opc) {
      case PGB_P_LAP: st[sp++] = lapv; break;
      case PGB_P_J0: st[sp++] = j0; break;
      case PGB_P_U: st[sp++] = arg ? (uv ? uv[arg - 1] : 0.0) : u; break;
      case PGB_P_SRC: st[sp++] = s[arg]; break;
      case PGB_P_CONST: st[sp++] = cst[arg]; break;
      case PGB_P_ADD: sp--; st[sp - 1] = st[sp - 1] + st[sp]; break;
      case PGB_P_SUB: sp--; st[sp - 1] = st[sp - 1] - st[sp]; break;
      case PGB_P_MUL: sp--; st[sp - 1] = st[sp - 1] * st[sp]; break;
      case PGB_P_DIV: sp--; st[sp - 1] = st[sp - 1] / st[sp]; break;
      case PGB_P_NEG: st[sp - 1] = -st[sp - 1]; break;
      default: break;
      }
   }
   return sp ? st[sp - 1] : 0.0;
}

int pgb_operator_eval(const pgb_operator *op, double lapv, double j0, double u, const double *s, double *L,
                      double *J)
{
   double sv[PGB_NSRC_MAX] = {0, 0, 0, 0};
   int k;
   if (!op) return 1;
   for (k = 0; k < op->d.nsrc; k++) sv[k] = s[k];
   if (L) *L = prog_eval_host(op->d.lcode, op->d.cst, lapv, j0, u, 0, sv);
   if (J) *J = prog_eval_host(op->d.jcode, op->d.cst, lapv, j0, u, 0, sv);
   return 0;
}

int pgb_operator_eval_vars(const pgb_operator *op, int var, double lapv, double j0, const double *uv,
                           const double *s, double *L, double *J)
{
   double sv[PGB_NSRC_MAX] = {0, 0, 0, 0};
   int k;
   if (!op || var < 0 || var >= PGB_NVAR_MAX || !uv) return 1;
   for (k = 0; k < op->d.nsrc; k++) sv[k] = s[k];
   if (L) *L = prog_eval_host(op->d.lcode, op->d.cst, lapv, j0, uv[var], uv, sv);
   if (J) *J = prog_eval_host(op->d.jcode, op->d.cst, lapv, j0, uv[var], uv, sv);
   return 0;
}

/* 1 when no derivative dL/du_k (k = 0..3, the names u0..u3) of the level
 * operator's program depends on lap or on a variable: the program's
 * values are followed abstractly (does it depend on the state, is its
 * derivative nonzero, does the derivative depend on the state) through the
 * rules of sums, products and quotients. The mixed form then computes its
 * coupling coefficients once per pgb_prepare instead of in every pass. */
int pgb_dop_couplings_fixed(const pgb_dop *d)
{
   int k;
   for (k = 0; k < PGB_NVAR_MAX; k++) {
      unsigned char dep[PGB_PROG_STACK + 1], dd[PGB_PROG_STACK + 1], ddep[PGB_PROG_STACK + 1];
      int q, sp = 0;
      for (q = 0; q < PGB_PROG_MAX && (d->lcode[q] & 15) != PGB_P_END; q++) {
         const int opc = d->lcode[q] & 15, arg = d->lcode[q] >> 4;
         if (opc == PGB_P_NEG) continue;
         if (opc >= PGB_P_ADD && opc <= PGB_P_DIV) {
            const int a = sp - 2, b = sp - 1;
            if (a < 0) return 0;
            ddep[a] = ddep[a] || ddep[b] || (opc == PGB_P_MUL && ((dd[a] && dep[b]) || (dd[b] && dep[a]))) ||
                      (opc == PGB_P_DIV && ((dd[a] && dep[b]) || dd[b]));
            dep[a] = dep[a] || dep[b];
            dd[a] = dd[a] || dd[b];
            sp--;
            continue;
         }
         if (sp > PGB_PROG_STACK) return 0;
         dep[sp] = opc == PGB_P_LAP || opc == PGB_P_U;
         dd[sp] = opc == PGB_P_U && arg == k + 1;
         ddep[sp] = 0;
         sp++;
      }
      if (sp > 0 && ddep[sp - 1]) return 0;
   }
   return 1;
}

/* 1 when the value of the operator's dL/du program depends neither on
 * lap nor on a variable (only on j0, the sources and constants): the
 * mixed form then computes its Jacobian term once per pgb_prepare too */
int pgb_dop_jac_fixed(const pgb_dop *d)
{
   int q;
   for (q = 0; q < PGB_PROG_MAX && (d->jcode[q] & 15) != PGB_P_END; q++)
      if ((d->jcode[q] & 15) == PGB_P_LAP || (d->jcode[q] & 15) == PGB_P_U) return 0;
   return 1;
}

/* 1 + the highest variable index an operator names (u0..u3), 0 if none */
int pgb_operator_vars(const pgb_operator *op)
{
   int q, n = 0;
   const unsigned char *codes[2] = {op->d.lcode, op->d.jcode};
   for (int c = 0; c < 2; c++)
      for (q = 0; q < PGB_PROG_MAX && (codes[c][q] & 15) != PGB_P_END; q++)
         if ((codes[c][q] & 15) == PGB_P_U && (codes[c][q] >> 4) > n) n = codes[c][q] >> 4;
   return n;
}

