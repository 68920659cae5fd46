/*
 * Launch geometry shared by the op-list kernels (sync copies, restrictions,
 * interpolations) of both precision forms. CUDA-only header.
 */
#ifndef PGB_OPGRID_CUH
#define PGB_OPGRID_CUH

#include "pgb_dev.h"

/* Op-list kernels run one op per blockIdx.z. Copies and restrictions walk
 * the op's (i,j) planes (blockIdx.y = k, 32-bit index arithmetic);
 * interpolations walk its x-rows (blockIdx.y = (j,k) row) so that the
 * box-edge points sit at fixed lanes. */
#define OP_PLANES(ni, nj, nk, ...)                                                    \
   for (int c = blockIdx.y; c < (nk); c += gridDim.y)                                \
      for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < (ni) * (nj);            \
           q += gridDim.x * blockDim.x) {                                             \
         const int a = q % (ni), bb = q / (ni);                                       \
         __VA_ARGS__                                                                  \
      }

/* A block as a kernel body sees it: a CTA of a standalone launch, or one
 * work item of a step of the small-level kernel (k_tail in
 * pgb_kernels32.cu), which runs the same bodies over a virtual grid. lt and
 * nt are the thread's linear index and the threads per block; the 32 x 8
 * tile bodies use threadIdx.x/y directly (k_tail has that shape). */
struct vblk {
   int x, y, z, gx, gy, gz, lt, nt;
};

__device__ __forceinline__ vblk hw_blk()
{
   vblk v;
   v.x = blockIdx.x;
   v.y = blockIdx.y;
   v.z = blockIdx.z;
   v.gx = gridDim.x;
   v.gy = gridDim.y;
   v.gz = gridDim.z;
   v.lt = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
   v.nt = blockDim.x * blockDim.y * blockDim.z;
   return v;
}

/* OP_PLANES over a vblk */
#define OP_PLANES_V(vb, ni, nj, nk, ...)                                              \
   for (int c = (vb).y; c < (nk); c += (vb).gy)                                      \
      for (int q = (vb).x * (vb).nt + (vb).lt; q < (ni) * (nj); q += (vb).gx * (vb).nt) { \
         const int a = q % (ni), bb = q / (ni);                                       \
         __VA_ARGS__                                                                  \
      }

/* launch geometry of a batch of ops: planes (copy, restrict) or x-rows
 * (interp); grid z = ops of the batch */
template <class T> static inline void plane_grid(const T *o, int n, dim3 &g)
{
   long mp = 1;
   int mk = 1;
   for (int i = 0; i < n; i++) {
      long p = (long)o[i].ni * o[i].nj;
      if (p > mp) mp = p;
      if (o[i].nk > mk) mk = o[i].nk;
   }
   long gx = (mp + 255) / 256;
   g = dim3((unsigned)(gx > 1024 ? 1024 : gx), (unsigned)(mk > 65535 ? 65535 : mk), (unsigned)n);
}

static inline void row_grid(const pgb_interp_op *o, int n, dim3 &g)
{
   int mx = 1;
   long mr = 1;
   for (int i = 0; i < n; i++) {
      long r = (long)o[i].njb * o[i].nkb;
      if (r > mr) mr = r;
      if (o[i].nib > mx) mx = o[i].nib;
   }
   int gx = (mx + 511) / 512;
   g = dim3((unsigned)gx, (unsigned)(mr > 65535 ? 65535 : mr), (unsigned)n);
}

#endif
