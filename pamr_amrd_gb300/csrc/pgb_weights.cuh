/*
 * The FP64 transfer arithmetic shared by both kernel files: the division by a
 * known divisor, 1-based box indexing, the half- and full-weighting stencils
 * of the restriction (and its FP32 residual form), and the bodies of the
 * restriction and field clear. pgb_kernels64.cu runs them in its standalone
 * kernels, pgb_kernels32.cu inside the small-level kernel. Every product in
 * them is either exact (a power-of-two weight) or an explicit FMA/rounding
 * intrinsic, so they give the same bits whether or not the including file
 * lets the compiler contract multiply-adds. CUDA-only header.
 */
#ifndef PGB_WEIGHTS_CUH
#define PGB_WEIGHTS_CUH

#include "pgb_opgrid.cuh"

/* RN(x/d) for a divisor whose correctly rounded reciprocal r = RN(1/d) is
 * known. q0 = RN(x*r) is within two ulps of x/d; one FMA correction step
 * q1 = RN(q0 + RN(x - q0*d)*r) leaves it within one ulp (faithful); with a
 * faithful quotient and r = RN(1/d), Markstein's theorem (P. Markstein, IBM
 * J. Res. Dev. 34, 1990; Muller et al., Handbook of Floating-Point
 * Arithmetic, 2018, sec. 4.7) makes the second step RN(x/d) exactly, barring
 * overflow and underflow. Five FP64 operations instead of a full division;
 * the GPU tests compare every result path with IEEE division. */
__device__ __forceinline__ double div_known(double x, double d, double r)
{
   double q = __dmul_rn(x, r);
   double e = __fma_rn(-q, d, x);
   q = __fma_rn(e, r, q);
   e = __fma_rn(-q, d, x);
   return __fma_rn(e, r, q);
}

/* point q of an ni x nj x nk segment -> (a,b,c) */
__device__ __forceinline__ void unflat(long q, int ni, int nj, int &a, int &bb, int &c)
{
   a = (int)(q % ni);
   long r = q / ni;
   bb = (int)(r % nj);
   c = (int)(r / nj);
}

__device__ __forceinline__ long lin(const pgb_dbox &b, int i1, int j1, int k1)
{
   /* 1-based (Fortran) indices */
   return (i1 - 1) + (long)b.n[0] * ((j1 - 1) + (long)b.n[1] * (k1 - 1));
}

/* The weights of the half- and full-weighting stencils are powers of two,
 * so w*u is exact and RN(acc + w*u) == fma(w, u, acc): the FMA forms below
 * give the Fortran sums bit for bit (same left-to-right order) with fewer
 * FP64 instructions. Divisions by 4, 8, 16 and 64 are exact products; the
 * division by 12 uses div_known. */
#define ACC(acc, w, v) __fma_rn((double)(w), (v), (acc))

/* dmhwr3d (src/m_util_r8.f:649-723), do_ex = 0, at fine point (i0,j0,k0) */
static __device__ double hwr(const double *u, int nx1, int ny1, int nz1, int i0, int j0, int k0)
{
   int w = 0;
   double sum = 0;
   long sy = nx1, sz = (long)nx1 * ny1;
   long p = (i0 - 1) + sy * (j0 - 1) + sz * (k0 - 1);
   if (i0 > 1 && i0 <= nx1 - 1) {
      w = w + 4;
      sum = ACC(sum + u[p - 1], 2, u[p]) + u[p + 1];
   }
   if (j0 > 1 && j0 <= ny1 - 1) {
      w = w + 4;
      sum = ACC(sum + u[p - sy], 2, u[p]) + u[p + sy];
   }
   if (k0 > 1 && k0 <= nz1 - 1) {
      w = w + 4;
      sum = ACC(sum + u[p - sz], 2, u[p]) + u[p + sz];
   }
   if (w == 12) return div_known(sum, 12.0, 1.0 / 12.0);
   if (w > 0) return sum * (w == 4 ? 0.25 : 0.125);
   return u[p];
}

/* dmfwr3d (src/m_util_r8.f:733-830), do_ex = 0, at fine point (i0,j0,k0):
 * the 27-, 9- or 3-point sum in the Fortran order (outer offset first) */
static __device__ double fwr(const double *u, int nx1, int ny1, int nz1, int i0, int j0, int k0)
{
   const long sy = nx1, sz = (long)nx1 * ny1;
   const long p = (i0 - 1) + sy * (j0 - 1) + sz * (k0 - 1);
   bool ii = i0 > 1 && i0 <= nx1 - 1, jj = j0 > 1 && j0 <= ny1 - 1, kk = k0 > 1 && k0 <= nz1 - 1;
   /* strides of the outer, middle and inner offsets of the sum */
   long s0, s1, s2;
   int n0, n1;
   double scale;
   if (ii && jj && kk) {
      s0 = sz; s1 = sy; s2 = 1; n0 = n1 = 3; scale = 1.0 / 64.0;
   } else if (ii && jj) {
      s0 = 0; s1 = sy; s2 = 1; n0 = 1; n1 = 3; scale = 1.0 / 16.0;
   } else if (jj && kk) {
      s0 = 0; s1 = sy; s2 = sz; n0 = 1; n1 = 3; scale = 1.0 / 16.0;
   } else if (ii && kk) {
      s0 = 0; s1 = 1; s2 = sz; n0 = 1; n1 = 3; scale = 1.0 / 16.0;
   } else if (ii || jj || kk) {
      s0 = 0; s1 = 0; s2 = ii ? 1 : (jj ? sy : sz); n0 = n1 = 1; scale = 0.25;
   } else
      return u[p];
   double acc = 0;
   bool first = true;
#pragma unroll
   for (int a = 0; a < 3; a++) {
      if (a >= n0) break;
      int da = n0 == 3 ? a - 1 : 0;
#pragma unroll
      for (int b = 0; b < 3; b++) {
         if (b >= n1) break;
         int db = n1 == 3 ? b - 1 : 0;
#pragma unroll
         for (int c = 0; c < 3; c++) {
            int dc = c - 1;
            double v = u[p + da * s0 + db * s1 + dc * s2];
            int w = (da == 0 ? 2 : 1) * (db == 0 ? 2 : 1) * (dc == 0 ? 2 : 1);
            if (n0 == 1) w >>= 1;
            if (n1 == 1) w >>= 1;
            acc = first ? (w == 1 ? v : (double)w * v) : ACC(acc, w, v);
            first = false;
         }
      }
   }
   return acc * scale;
}
#undef ACC

/* fwr of the residual in FP32 for the mixed form: the same weights and sums
 * over D, the FP32 copy of -res that the mixed form's residual pass leaves
 * at the points where it writes res (0 wherever res is 0). The restricted
 * residual only steers the coarse-grid correction, so FP32 is enough; the
 * FP64 residual of the finest level still decides convergence. */
static __device__ double fwr_d32(const float *dd, int wy, long wz, int nx1, int ny1, int nz1, int i0, int j0, int k0)
{
   const int sy = wy;
   const long sz = wz;   /* the FP32 arrays' padded pitches */
   const long p = (i0 - 1) + (long)sy * (j0 - 1) + sz * (k0 - 1);
   bool ii = i0 > 1 && i0 <= nx1 - 1, jj = j0 > 1 && j0 <= ny1 - 1, kk = k0 > 1 && k0 <= nz1 - 1;
   long s0, s1, s2;
   int n0, n1;
   float scale;
   if (ii && jj && kk) {
      s0 = sz; s1 = sy; s2 = 1; n0 = n1 = 3; scale = 1.f / 64.f;
   } else if (ii && jj) {
      s0 = 0; s1 = sy; s2 = 1; n0 = 1; n1 = 3; scale = 1.f / 16.f;
   } else if (jj && kk) {
      s0 = 0; s1 = sy; s2 = sz; n0 = 1; n1 = 3; scale = 1.f / 16.f;
   } else if (ii && kk) {
      s0 = 0; s1 = 1; s2 = sz; n0 = 1; n1 = 3; scale = 1.f / 16.f;
   } else if (ii || jj || kk) {
      s0 = 0; s1 = 0; s2 = ii ? 1 : (jj ? sy : sz); n0 = n1 = 1; scale = 0.25f;
   } else
      return -(double)dd[p];
   float acc = 0.f;
#pragma unroll
   for (int a = 0; a < 3; a++) {
      if (a >= n0) break;
      const int da = n0 == 3 ? a - 1 : 0;
#pragma unroll
      for (int b = 0; b < 3; b++) {
         if (b >= n1) break;
         const int db = n1 == 3 ? b - 1 : 0;
         const float wab = (float)((da == 0 ? 2 : 1) * (db == 0 ? 2 : 1) >> (n0 == 1 ? 1 : 0) >> (n1 == 1 ? 1 : 0));
         const float *r = dd + p + da * s0 + db * s1;
         acc = __fmaf_rn(wab, __fadd_rn(__fadd_rn(r[-s2], 2.f * r[0]), r[s2]), acc);
      }
   }
   return -(double)__fmul_rn(acc, scale);
}

/* local_transfer delta = +1 (src/transfer.c:1126-1149): per grid function
 * straight injection, half weighting or full weighting; res32 = 1 (mixed
 * form) takes the full weighting of the residual from its FP32 copy */
__device__ __forceinline__ void restrict_b(const vblk &vb, const pgb_dbox *boxes, const pgb_restrict_op *ops,
                                           int field_mask, int res32)
{
   const pgb_restrict_op o = ops[vb.z];
   const pgb_dbox &s = boxes[o.src_box];
   const pgb_dbox &d = boxes[o.dst_box];
   OP_PLANES_V(vb, o.ni, o.nj, o.nk, {
      const int i0 = o.i1 + a * o.irho, j0 = o.j1 + bb * o.irho, k0 = o.k1 + c * o.irho;
      const long pd = lin(d, o.i2 + a, o.j2 + bb, o.k2 + c);
      for (int f = 0; f < PGB_NF; f++) {
         const int op = o.op[f];
         if (!op || !((field_mask >> f) & 1)) continue;
         const double *u = s.f[f];
         double v;
         if (op == 1) v = u[lin(s, i0, j0, k0)];
         else if (op == 2) v = hwr(u, s.n[0], s.n[1], s.n[2], i0, j0, k0);
         else if (res32 && f == PGB_F_RES) v = fwr_d32(s.w32[PGB_W32_D], s.wy, s.wz, s.n[0], s.n[1], s.n[2], i0, j0, k0);
         else v = fwr(u, s.n[0], s.n[1], s.n[2], i0, j0, k0);
         d.f[f][pd] = v;
      }
   })
}

/* clear_MG_vars (amrd/mg.c:242-262): the fields of `mask` set to 0 on tile
 * vb.x of the level (32 x 8 threads, up to PGB_TZ planes each) */
__device__ __forceinline__ void clear_b(const vblk &vb, const pgb_dbox *boxes, const pgb_dlevel &lv, int mask)
{
   const pgb_tile tl = lv.tiles[vb.x];
   const pgb_dbox &b = boxes[tl.box];
   const int i = tl.i0 + threadIdx.x, j = tl.j0 + threadIdx.y;
   const int kz = lv.dim == 3 ? lv.tz : 1;
   if (i >= b.n[0] || j >= b.n[1]) return;
   for (int kk = 0; kk < kz; kk++) {
      const int k = tl.k0 + kk;
      if (k >= b.n[2]) break;
      const long p = i + (long)b.n[0] * (j + (long)b.n[1] * k);
      for (int f = 0; f < PGB_NF; f++)
         if ((mask >> f) & 1) b.f[f][p] = 0;
   }
}

#endif
