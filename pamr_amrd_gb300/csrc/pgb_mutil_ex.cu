/*
 * Excision-aware m_util_r8 kernels of libpamr_gb300 (sm_103a), bit-exact
 * with the Fortran (compiled with -fmad=false; same expression order):
 *   dmhwr3d with do_ex = 1       src/m_util_r8.f:649-723
 *   dmfwr3d_ex                   src/m_util_r8.f:835-949
 *   dminterp3d with do_ex = 1    src/m_util_r8.f:473-637 over
 *   dvi2q1d_ex / dvi4q1d_ex      src/m_util_r8.f:368-421, 153-319
 *   init_chrt / and_chrt         src/m_util_r8.f:426-456
 * chr1 is the mask of u1 (a double per point; a point is excised when its
 * value equals ex). The interpolation overwrites parts of u2's excised zone,
 * as the Fortran does. Its 1-D passes are sequential along a line (the
 * extrapolation into the excised zone feeds the stencils that follow), so
 * one thread runs one line, and the i-, j- and k-line phases are separate
 * launches in the Fortran's order. The per-line mask chrt is evaluated on the
 * fly from chr1 instead of being staged in a scratch array.
 */
#include <cuda_runtime.h>
#include <stdio.h>
#include "pgb_dev.h"

static __thread char g_err_ex[256];
static unsigned long long g_launches_ex = 0;

extern "C" unsigned long long pgb_dev_launches_ex(void) { return g_launches_ex; }
extern "C" const char *pgb_dev_error_ex(void) { return g_err_ex; }

static int check_ex(const char *what)
{
   g_launches_ex++;
   cudaError_t e = cudaGetLastError();
   if (e != cudaSuccess) {
      snprintf(g_err_ex, sizeof(g_err_ex), "%s: %s", what, cudaGetErrorString(e));
      pgb_note_error(g_err_ex);
      return 1;
   }
   return 0;
}

static int arg_error(const char *msg)
{
   snprintf(g_err_ex, sizeof(g_err_ex), "%s", msg);
   pgb_note_error(g_err_ex);
   return 12;
}

/* 1-based Fortran element v(i) */
#define F1(v, i) (v)[(i)-1]

/* Excision test of a line mask: chrt(idx) == ex. With one contributing
 * chr1 line (nb = 1) this is the raw compare on chr1 memory, as the Fortran
 * reads chr1 (or the init_chrt copy of it) through a 1-D dummy array: an
 * index past the line reads the neighbouring memory of chr1, which is
 * followed here as long as it stays inside chr1 (outside it, not excised).
 * With more lines (and_chrt) a point is excised only where every
 * contributing value is ex; indices outside 1..n, where the Fortran's
 * scratch array holds no defined value, count as not excised. */
struct LineMask {
   const double *b[4];
   const double *lo;   /* chr1 */
   long total;         /* points of chr1 */
   int nb;
   long s;             /* stride between consecutive mask entries in chr1 */
   int n;
   double ex;
   __device__ bool operator()(int idx) const
   {
      const long o = (long)(idx - 1) * s;
      if (nb == 1) {
         const long f = (long)(b[0] - lo) + o;
         return f >= 0 && f < total && lo[f] == ex;
      }
      if (idx < 1 || idx > n) return false;
      for (int q = 0; q < nb; q++)
         if (!(b[q][o] == ex)) return false;
      return true;
   }
};

/* dvi2q1d_ex; v1 and v2 alias (dminterp3d passes the same line) */
__device__ void dvi2q1d_ex(double *v1, double *v2, int i1, int i2, int n1, int n, int irho, int s1,
                           int s2, const LineMask &chr, int i3, int s3)
{
   int i, j, i10, i30;
   double c0, c1, sg;
   for (i = 1; i <= n; i++) {
      i10 = (i - 1) * s1 + i1;
      i30 = (i - 1) * s3 + i3;
      if (chr(i30)) {
         if (i10 > 3 * s1 && !chr(i30 - s3) && !chr(i30 - 2 * s3) && !chr(i30 - 3 * s3))
            F1(v1, i10) = 3 * (F1(v1, i10 - s1) - F1(v1, i10 - 2 * s1)) + F1(v1, i10 - 3 * s1);
         else if (i10 <= (n1 - 3 * s1) && !chr(i30 + s3) && !chr(i30 + 2 * s3) && !chr(i30 + 3 * s3))
            F1(v1, i10) = 3 * (F1(v1, i10 + s1) - F1(v1, i10 + 2 * s1)) + F1(v1, i10 + 3 * s1);
         else if (i10 > 2 * s1 && !chr(i30 - s3) && !chr(i30 - 2 * s3))
            F1(v1, i10) = 2 * F1(v1, i10 - s1) - F1(v1, i10 - 2 * s1);
         else if (i10 <= (n1 - 2 * s1) && !chr(i30 + s3) && !chr(i30 + 2 * s3))
            F1(v1, i10) = 2 * F1(v1, i10 + s1) - F1(v1, i10 + 2 * s1);
         else if (i10 > s1 && !chr(i30 - s3))
            F1(v1, i10) = F1(v1, i10 - s1);
         else if (i10 <= (n1 - s1) && !chr(i30 + s3))
            F1(v1, i10) = F1(v1, i10 + s1);
      }
      F1(v2, irho * (i - 1) * s2 + i2) = F1(v1, i10);
   }
   for (j = 1; j <= irho - 1; j++) {
      sg = (j * 1.0) / irho;
      c0 = 1 - sg;
      c1 = sg;
      for (i = 0; i <= n - 2; i++) {
         i10 = (irho * i + j) * s2 + i2;
         F1(v2, i10) = c0 * F1(v1, i * s1 + i1) + c1 * F1(v1, (i + 1) * s1 + i1);
      }
   }
}

__device__ __forceinline__ void cubic_cf(double sg, double &c0, double &c1, double &c2, double &c3)
{
   const double HALF = 0.5, MHALF = -0.5, SIXTH = 0.16666666666666667, MSIXTH = -0.16666666666666667;
   c0 = MSIXTH * (sg - 1.0) * (sg - 2.0) * (sg - 3.0);
   c1 = HALF * sg * (sg - 2.0) * (sg - 3.0);
   c2 = MHALF * sg * (sg - 1.0) * (sg - 3.0);
   c3 = SIXTH * sg * (sg - 1.0) * (sg - 2.0);
}

/* dvi4q1d_ex (irho <= 20, checked on the host) */
__device__ void dvi4q1d_ex(double *v1, double *v2, int i1, int i2, int n1, int n, int irho, int s1,
                           int s2, const LineMask &chr, int i3, int s3)
{
   int i, j, cn, j0, i1s, i1e, i10, i30;
   bool init_2;
   double c0, c1, c2, c3;
   i = 3;
   i1s = i1;
   while (i > 0 && i1s > s1) {
      i1s = i1s - s1;
      i = i - 1;
   }
   i = 3;
   i1e = i1 + (n - 1) * s1;
   while (i > 0 && i1e < (n1 - s1)) {
      i1e = i1e + s1;
      i = i - 1;
   }
   cn = 0;
   init_2 = false;
   for (i = i1s; i <= i1e; i += s1) {
      if (chr((i - i1) * s3 / s1 + i3) || i == i1e) {
         if (cn > 0 && cn < 4) init_2 = true;
         else cn = 0;
      } else
         cn = cn + 1;
   }
   if (init_2) dvi2q1d_ex(v1, v2, i1, i2, n1, n, irho, s1, s2, chr, i3, s3);
#define CH(off) chr(i3 + s3 * ((off) - i1) / s1)
   for (i = i1s; i <= i1e; i += s1) {
      if (CH(i)) {
         if (i >= (i1s + 3 * s1) && !CH(i - s1) && !CH(i - 2 * s1) && !CH(i - 3 * s1)) {
            if (i >= (i1s + 4 * s1) && !CH(i - 4 * s1))
               F1(v1, i) = 4 * (F1(v1, i - s1) + F1(v1, i - 3 * s1)) - 6 * F1(v1, i - 2 * s1) -
                           F1(v1, i - 4 * s1);
            else
               F1(v1, i) = 3 * (F1(v1, i - s1) - F1(v1, i - 2 * s1)) + F1(v1, i - 3 * s1);
         } else if (i <= (i1e - 3 * s1) && !CH(i + s1) && !CH(i + 2 * s1) && !CH(i + 3 * s1)) {
            if (i <= (i1s - 4 * s1) && !CH(i + 4 * s1))   /* i1s as in the Fortran */
               F1(v1, i) = 4 * (F1(v1, i + s1) + F1(v1, i + 3 * s1)) - 6 * F1(v1, i + 2 * s1) -
                           F1(v1, i + 4 * s1);
            else
               F1(v1, i) = 3 * (F1(v1, i + s1) - F1(v1, i + 2 * s1)) + F1(v1, i + 3 * s1);
         }
      }
      if (i >= i1 && i <= (i1 + (n - 1) * s1)) F1(v2, irho * ((i - i1) / s1) * s2 + i2) = F1(v1, i);
   }
#undef CH
   for (i = 1; i <= n - 1; i++) {   /* left boundary cells */
      i10 = (i - 1) * s1 + i1;
      i30 = (i - 1) * s3 + i3;
      j0 = (i - 1) * irho * s2 + i2;
      if (i10 <= (i1e - 3 * s1) && !chr(i30 + s3) && !chr(i30 + 2 * s3) &&
          ((i == 1 && i10 == i1s) || (i10 >= (i1s + s1) && !chr(i30) && chr(i30 - s3)) || chr(i30)))
         for (j = 1; j <= irho - 1; j++) {
            cubic_cf((j * 1.0) / irho, c0, c1, c2, c3);
            F1(v2, j * s2 + j0) = c0 * F1(v1, i10) + c1 * F1(v1, s1 + i10) + c2 * F1(v1, 2 * s1 + i10) +
                                  c3 * F1(v1, 3 * s1 + i10);
         }
   }
   for (i = 1; i <= n - 1; i++) {   /* right boundary cells */
      i10 = (i - 1) * s1 + i1;
      i30 = (i - 1) * s3 + i3;
      j0 = (i - 1) * irho * s2 + i2;
      if (i10 >= (i1s + 2 * s1) && !chr(i30 - s3) &&
          ((i == (n - 1) && i10 == (i1e - s1)) || (i10 <= (i1e - s1) && !chr(i30) && chr(i30 + s3))))
         for (j = 1; j <= irho - 1; j++) {
            cubic_cf(2.0 + (j * 1.0) / irho, c0, c1, c2, c3);
            F1(v2, j * s2 + j0) = c0 * F1(v1, i10 - 2 * s1) + c1 * F1(v1, i10 - s1) + c2 * F1(v1, i10) +
                                  c3 * F1(v1, i10 + s1);
         }
   }
   for (i = 1; i <= n; i++) {   /* interior */
      i10 = (i - 1) * s1 + i1;
      i30 = (i - 1) * s3 + i3;
      j0 = (i - 1) * irho * s2 + i2;
      if (!chr(i30) && i10 >= (i1s + s1) && !chr(i30 - s3) && i10 <= (i1e - 2 * s1) && !chr(i30 + s3))
         for (j = 1; j <= irho - 1; j++) {
            cubic_cf(1.0 + (j * 1.0) / irho, c0, c1, c2, c3);
            F1(v2, j0 + j * s2) = c0 * F1(v1, i10 - s1) + c1 * F1(v1, i10) + c2 * F1(v1, i10 + s1) +
                                  c3 * F1(v1, i10 + 2 * s1);
         }
   }
}

typedef struct {
   int nx1, ny1, nz1, nx2, ny2, nz2, i1, j1, k1, i2, j2, k2, ni, nj, nk, si1, sj1, sk1;
   int irho, jrho, krho, ord;
} mx_args;

__device__ __forceinline__ const double *chr_at(const double *chr1, const mx_args &a, int i, int j, int k)
{
   return chr1 + (i - 1) + (long)a.nx1 * ((j - 1) + (long)a.ny1 * (k - 1));
}

/* phase 1: the i-lines through the anchor rows (j, k of the segment) */
__global__ void k_mex_ilines(double *u2, const double *chr1, double ex, mx_args a)
{
   const int q = blockIdx.x * blockDim.x + threadIdx.x;
   if (q >= a.nj * a.nk) return;
   const int jj = q % a.nj, kk = q / a.nj;
   const int j = a.j2 + jj * a.jrho, k = a.k2 + kk * a.krho;
   double *line = u2 + (long)a.nx2 * ((j - 1) + (long)a.ny2 * (k - 1));
   LineMask m;
   m.b[0] = chr_at(chr1, a, 1, a.j1 + a.sj1 * (j - a.j2) / a.jrho, a.k1 + a.sk1 * (k - a.k2) / a.krho);
   m.nb = 1;
   m.s = 1;
   m.n = a.nx1;
   m.ex = ex;
   m.lo = chr1;
   m.total = (long)a.nx1 * a.ny1 * a.nz1;
   if (a.ord == 2) dvi2q1d_ex(line, line, a.i2, a.i2, a.nx2, a.ni, a.irho, a.irho, 1, m, a.i1, a.si1);
   else dvi4q1d_ex(line, line, a.i2, a.i2, a.nx2, a.ni, a.irho, a.irho, 1, m, a.i1, a.si1);
}

/* phase 2: the j-lines at every i of the segment, anchor k */
__global__ void k_mex_jlines(double *u2, const double *chr1, double ex, mx_args a)
{
   const int ni2 = (a.ni - 1) * a.irho + 1;
   const int q = blockIdx.x * blockDim.x + threadIdx.x;
   if (q >= ni2 * a.nk) return;
   const int i = a.i2 + q % ni2, k = a.k2 + (q / ni2) * a.krho;
   const int ci = a.i1 + a.si1 * ((i - a.i2) / a.irho), ck = a.k1 + a.sk1 * ((k - a.k2) / a.krho);
   LineMask m;
   m.b[0] = chr_at(chr1, a, ci, 1, ck);
   m.nb = 1;
   if ((i - a.i2) % a.irho != 0) m.b[m.nb++] = chr_at(chr1, a, a.i1 + a.si1 * ((i - a.i2) / a.irho + 1), 1, ck);
   m.s = a.nx1;
   m.n = a.ny1;
   m.ex = ex;
   m.lo = chr1;
   m.total = (long)a.nx1 * a.ny1 * a.nz1;
   double *line = u2 + (i - 1) + (long)a.nx2 * a.ny2 * (k - 1);
   const int st = 1 + (a.j2 - 1) * a.nx2, n12 = a.nx2 * (a.ny2 - 1) + 1;
   if (a.ord == 2) dvi2q1d_ex(line, line, st, st, n12, a.nj, a.jrho, a.jrho * a.nx2, a.nx2, m, a.j1, a.sj1);
   else dvi4q1d_ex(line, line, st, st, n12, a.nj, a.jrho, a.jrho * a.nx2, a.nx2, m, a.j1, a.sj1);
}

/* phase 3: the k-lines at every (i, j) of the segment */
__global__ void k_mex_klines(double *u2, const double *chr1, double ex, mx_args a)
{
   const int ni2 = (a.ni - 1) * a.irho + 1, nj2 = (a.nj - 1) * a.jrho + 1;
   const int q = blockIdx.x * blockDim.x + threadIdx.x;
   if (q >= ni2 * nj2) return;
   const int i = a.i2 + q % ni2, j = a.j2 + q / ni2;
   const int ci = a.i1 + a.si1 * ((i - a.i2) / a.irho), cj = a.j1 + a.sj1 * ((j - a.j2) / a.jrho);
   const bool oi = (i - a.i2) % a.irho != 0, oj = (j - a.j2) % a.jrho != 0;
   LineMask m;
   m.b[0] = chr_at(chr1, a, ci, cj, 1);
   m.nb = 1;
   if (oi) m.b[m.nb++] = chr_at(chr1, a, ci + a.si1, cj, 1);
   if (oj) m.b[m.nb++] = chr_at(chr1, a, ci, cj + a.sj1, 1);
   if (oi && oj) m.b[m.nb++] = chr_at(chr1, a, ci + a.si1, cj + a.sj1, 1);
   m.s = (long)a.nx1 * a.ny1;
   m.n = a.nz1;
   m.ex = ex;
   m.lo = chr1;
   m.total = (long)a.nx1 * a.ny1 * a.nz1;
   double *line = u2 + (i - 1) + (long)a.nx2 * (j - 1);
   const int st = (a.k2 - 1) * a.nx2 * a.ny2 + 1, n12 = a.nx2 * a.ny2 * (a.nz2 - 1) + 1;
   if (a.ord == 2)
      dvi2q1d_ex(line, line, st, st, n12, a.nk, a.krho, a.krho * a.nx2 * a.ny2, a.nx2 * a.ny2, m, a.k1, a.sk1);
   else
      dvi4q1d_ex(line, line, st, st, n12, a.nk, a.krho, a.krho * a.nx2 * a.ny2, a.nx2 * a.ny2, m, a.k1, a.sk1);
}

/* dmcopy3d of the anchors (u1 segment with strides s*1 -> u2 with strides rho) */
__global__ void k_mex_copy(const double *u1, double *u2, mx_args a)
{
   const long npts = (long)a.ni * a.nj * a.nk;
   for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < npts; q += (long)gridDim.x * blockDim.x) {
      const int i = (int)(q % a.ni), j = (int)((q / a.ni) % a.nj), k = (int)(q / ((long)a.ni * a.nj));
      const int ii = a.i1 + i * a.si1, jj = a.j1 + j * a.sj1, kk = a.k1 + k * a.sk1;
      const int io = a.i2 + i * a.irho, jo = a.j2 + j * a.jrho, ko = a.k2 + k * a.krho;
      u2[(io - 1) + (long)a.nx2 * ((jo - 1) + (long)a.ny2 * (ko - 1))] =
         u1[(ii - 1) + (long)a.nx1 * ((jj - 1) + (long)a.ny1 * (kk - 1))];
   }
}

static int grid1(long n) { return (int)((n + 127) / 128); }

extern "C" int pgb_dminterp3d_ex(const double *u1, double *u2, int nx1, int ny1, int nz1, int nx2,
                                 int ny2, int nz2, int i1, int j1, int k1, int i2, int j2, int k2,
                                 int ni, int nj, int nk, int si1, int sj1, int sk1, int irho, int jrho,
                                 int krho, int ord, const double *chr1, double ex, void *stream)
{
   mx_args a = {nx1, ny1, nz1, nx2, ny2, nz2, i1, j1, k1, i2, j2, k2, ni, nj, nk,
                si1, sj1, sk1, irho, jrho, krho, ord};
   cudaStream_t st = (cudaStream_t)stream;
   if (i1 < 1 || (i1 + ni - 1) * si1 > nx1) return 0;
   if (i2 < 1 || (i2 + (ni - 1) * irho) > nx2) return 0;
   if (j1 < 1 || (j1 + nj - 1) * sj1 > ny1) return 0;
   if (j2 < 1 || (j2 + (nj - 1) * jrho) > ny2) return 0;
   if (k1 < 1 || (k1 + nk - 1) * sk1 > nz1) return 0;
   if (k2 < 1 || (k2 + (nk - 1) * krho) > nz2) return 0;
   if (ord != 2 && ord != 4) return arg_error("dminterp3d: only ord=2,4 supported");
   if (nx1 > 3000 || ny1 > 3000 || nz1 > 3000) return arg_error("dminterp3d: nmax too small");
   if (ord == 4 && (irho > 20 || jrho > 20 || krho > 20))
      return arg_error("dvi4q1d_ex : irho expected to be less than 20");
   {
      long n = (long)ni * nj * nk, g = (n + 127) / 128;
      k_mex_copy<<<(int)(g > 4096 ? 4096 : g), 128, 0, st>>>(u1, u2, a);
      if (check_ex("dminterp3d_ex copy")) return 11;
   }
   k_mex_ilines<<<grid1((long)nj * nk), 128, 0, st>>>(u2, chr1, ex, a);
   if (check_ex("dminterp3d_ex i-lines")) return 11;
   if (nj == 1 && nk == 1) return 0;
   k_mex_jlines<<<grid1(((long)(ni - 1) * irho + 1) * nk), 128, 0, st>>>(u2, chr1, ex, a);
   if (check_ex("dminterp3d_ex j-lines")) return 11;
   if (nk == 1) return 0;
   k_mex_klines<<<grid1(((long)(ni - 1) * irho + 1) * ((long)(nj - 1) * jrho + 1)), 128, 0, st>>>(u2, chr1, ex, a);
   if (check_ex("dminterp3d_ex k-lines")) return 11;
   return 0;
}

typedef struct {
   int nx1, ny1, nz1, nx2, ny2, nz2, i1, j1, k1, i2, j2, k2, ni, nj, nk;
   int si1, sj1, sk1, si2, sj2, sk2;
} mr_args;

#define UU(a_, b_, c_) u1[((a_)-1) + (long)a.nx1 * (((b_)-1) + (long)a.ny1 * ((c_)-1))]
#define CC(a_, b_, c_) chr1[((a_)-1) + (long)a.nx1 * (((b_)-1) + (long)a.ny1 * ((c_)-1))]

/* dmhwr3d with do_ex = 1 */
__global__ void k_mex_hwr(const double *u1, double *u2, const double *chr1, double ex, mr_args a)
{
   const long npts = (long)a.ni * a.nj * a.nk;
   for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < npts; q += (long)gridDim.x * blockDim.x) {
      const int i = (int)(q % a.ni), j = (int)((q / a.ni) % a.nj), k = (int)(q / ((long)a.ni * a.nj));
      const int i0 = a.i1 + i * a.si1, j0 = a.j1 + j * a.sj1, k0 = a.k1 + k * a.sk1;
      int w = 0;
      double sum = 0;
      if (i0 > 1 && i0 <= (a.nx1 - 1) && CC(i0 - 1, j0, k0) != ex && CC(i0, j0, k0) != ex &&
          CC(i0 + 1, j0, k0) != ex) {
         w = w + 4;
         sum = sum + UU(i0 - 1, j0, k0) + 2 * UU(i0, j0, k0) + UU(i0 + 1, j0, k0);
      }
      if (j0 > 1 && j0 <= (a.ny1 - 1) && CC(i0, j0 - 1, k0) != ex && CC(i0, j0, k0) != ex &&
          CC(i0, j0 + 1, k0) != ex) {
         w = w + 4;
         sum = sum + UU(i0, j0 - 1, k0) + 2 * UU(i0, j0, k0) + UU(i0, j0 + 1, k0);
      }
      if (k0 > 1 && k0 <= (a.nz1 - 1) && CC(i0, j0, k0 - 1) != ex && CC(i0, j0, k0) != ex &&
          CC(i0, j0, k0 + 1) != ex) {
         w = w + 4;
         sum = sum + UU(i0, j0, k0 - 1) + 2 * UU(i0, j0, k0) + UU(i0, j0, k0 + 1);
      }
      double v;
      if (CC(i0, j0, k0) == ex) v = 0;
      else if (w > 0) v = sum / w;
      else v = UU(i0, j0, k0);
      u2[(a.i2 + i * a.si2 - 1) + (long)a.nx2 * ((a.j2 + j * a.sj2 - 1) + (long)a.ny2 * (a.k2 + k * a.sk2 - 1))] = v;
   }
}

/* w3d(a,b,c) of dmfwr3d_ex through its column-major storage; an offset past
 * the 27 entries (reachable only through the Fortran's w3d(i,1,k) in the
 * k-only branch) counts as 0 */
__device__ __forceinline__ int w3d(int p, int r, int c)
{
   const int o = (p - 1) + 3 * (r - 1) + 9 * (c - 1);
   if (o < 0 || o >= 27) return 0;
   const int ip = o % 3, jr = (o / 3) % 3, kc = o / 9;
   return (ip == 1 ? 2 : 1) * (jr == 1 ? 2 : 1) * (kc == 1 ? 2 : 1);
}

/* dmfwr3d_ex */
__global__ void k_mex_fwr(const double *u1, double *u2, const double *chr1, double ex, mr_args a)
{
   const long npts = (long)a.ni * a.nj * a.nk;
   for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < npts; q += (long)gridDim.x * blockDim.x) {
      const int i = (int)(q % a.ni), j = (int)((q / a.ni) % a.nj), k = (int)(q / ((long)a.ni * a.nj));
      const int i0 = a.i1 + i * a.si1, j0 = a.j1 + j * a.sj1, k0 = a.k1 + k * a.sk1;
      const int im = i0 - 1, jm = j0 - 1, km = k0 - 1, ip = i0 + 1, jp = j0 + 1, kp = k0 + 1;
      const bool ii = i0 > 1 && i0 <= (a.nx1 - 1), jj = j0 > 1 && j0 <= (a.ny1 - 1),
                 kk = k0 > 1 && k0 <= (a.nz1 - 1);
      double sum = 0;
      int w = 0;
      if (ii && jj && kk) {
         for (int x = im; x <= ip; x++)
            for (int y = jm; y <= jp; y++)
               for (int z = km; z <= kp; z++)
                  if (CC(x, y, z) != ex) {
                     sum = sum + w3d(x - im + 1, y - jm + 1, z - km + 1) * UU(x, y, z);
                     w = w + w3d(x - im + 1, y - jm + 1, z - km + 1);
                  }
      } else if (ii && jj) {
         for (int x = im; x <= ip; x++)
            for (int y = jm; y <= jp; y++)
               if (CC(x, y, k0) != ex) {
                  sum = sum + w3d(x - im + 1, y - jm + 1, 1) * UU(x, y, k0);
                  w = w + w3d(x - im + 1, y - jm + 1, 1);
               }
      } else if (jj && kk) {
         for (int y = jm; y <= jp; y++)
            for (int z = km; z <= kp; z++)
               if (CC(i0, y, z) != ex) {
                  sum = sum + w3d(1, y - jm + 1, z - km + 1) * UU(i0, y, z);
                  w = w + w3d(1, y - jm + 1, z - km + 1);
               }
      } else if (ii && kk) {
         for (int x = im; x <= ip; x++)
            for (int z = km; z <= kp; z++)
               if (CC(x, j0, z) != ex) {
                  sum = sum + w3d(x - im + 1, 1, z - km + 1) * UU(x, j0, z);
                  w = w + w3d(x - im + 1, 1, z - km + 1);
               }
      } else if (ii) {
         for (int x = im; x <= ip; x++)
            if (CC(x, j0, k0) != ex) {
               sum = sum + w3d(x - im + 1, 1, 1) * UU(x, j0, k0);
               w = w + w3d(x - im + 1, 1, 1);
            }
      } else if (jj) {
         for (int y = jm; y <= jp; y++)
            if (CC(i0, y, k0) != ex) {
               sum = sum + w3d(1, y - jm + 1, 1) * UU(i0, y, k0);
               w = w + w3d(1, y - jm + 1, 1);
            }
      } else if (kk) {
         for (int z = km; z <= kp; z++)
            if (CC(i0, j0, z) != ex) {
               sum = sum + w3d(1, 1, z - km + 1) * UU(i0, j0, z);
               w = w + w3d(i + 1, 1, z - km + 1);   /* the Fortran's w3d(i,1,k), i 1-based */
            }
      } else {
         sum = UU(i0, j0, k0);
         w = 1;
      }
      const double v = (w == 0 || CC(i0, j0, k0) == ex) ? 0.0 : sum / w;
      u2[(a.i2 + i * a.si2 - 1) + (long)a.nx2 * ((a.j2 + j * a.sj2 - 1) + (long)a.ny2 * (a.k2 + k * a.sk2 - 1))] = v;
   }
}
#undef UU
#undef CC

static bool mr_in_range(const mr_args &a)
{
   if (a.i1 < 1 || (a.i1 + (a.ni - 1) * a.si1) > a.nx1) return false;
   if (a.i2 < 1 || (a.i2 + (a.ni - 1) * a.si2) > a.nx2) return false;
   if (a.j1 < 1 || (a.j1 + (a.nj - 1) * a.sj1) > a.ny1) return false;
   if (a.j2 < 1 || (a.j2 + (a.nj - 1) * a.sj2) > a.ny2) return false;
   if (a.k1 < 1 || (a.k1 + (a.nk - 1) * a.sk1) > a.nz1) return false;
   if (a.k2 < 1 || (a.k2 + (a.nk - 1) * a.sk2) > a.nz2) return false;
   return true;
}

#define MR_SIG                                                                               \
   const double *u1, double *u2, int nx1, int ny1, int nz1, int nx2, int ny2, int nz2, int i1, \
      int j1, int k1, int i2, int j2, int k2, int ni, int nj, int nk, int si1, int sj1, int sk1, \
      int si2, int sj2, int sk2, const double *chr1, double ex, void *stream
#define MR_ARGS                                                                              \
   mr_args a = {nx1, ny1, nz1, nx2, ny2, nz2, i1, j1, k1, i2, j2, k2, ni, nj, nk,            \
                si1, sj1, sk1, si2, sj2, sk2};                                               \
   long n = (long)ni * nj * nk, g = (n + 127) / 128;                                         \
   if (!mr_in_range(a) || n <= 0) return 0;                                                  \
   if (g > 4096) g = 4096;

extern "C" int pgb_dmhwr3d_ex(MR_SIG)
{
   MR_ARGS
   k_mex_hwr<<<(int)g, 128, 0, (cudaStream_t)stream>>>(u1, u2, chr1, ex, a);
   return check_ex("dmhwr3d_ex") ? 11 : 0;
}

extern "C" int pgb_dmfwr3d_ex(MR_SIG)
{
   MR_ARGS
   k_mex_fwr<<<(int)g, 128, 0, (cudaStream_t)stream>>>(u1, u2, chr1, ex, a);
   return check_ex("dmfwr3d_ex") ? 11 : 0;
}
