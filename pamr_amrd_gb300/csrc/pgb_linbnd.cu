/*
 * Linear approach to the boundaries, linbnd3d (src/m_util_r8.f:1957-2252),
 * on a device array, bit-exact with the Fortran (compiled with
 * -fmad=false). The Fortran is a fixed sequence of statements, each a loop
 * over points of one face, edge or corner whose values are means of their
 * neighbours across the boundary; a later statement may read what an
 * earlier one wrote (small extents, edges next to faces). One CTA runs the
 * statements in the Fortran's order with a barrier after each, its threads
 * sharing each statement's loop (a statement's points are independent).
 * As in the Fortran, the corner conditions read (A .and. B) .or. (all .and.
 * X): the excision test X applies only when all faces are selected; for
 * which_bnd = 3 the Fortran's pf is undefined, here it matches no face.
 */
#include <cuda_runtime.h>
#include <stdio.h>
#include "pgb_dev.h"

static __thread char g_err_lb[256];
static unsigned long long g_launches_lb = 0;

extern "C" unsigned long long pgb_dev_launches_lb(void) { return g_launches_lb; }

static int fail_lb(const char *msg, int rc)
{
   snprintf(g_err_lb, sizeof(g_err_lb), "%s", msg);
   pgb_note_error(g_err_lb);
   return rc;
}

#define LB_THREADS 1024

__global__ void __launch_bounds__(LB_THREADS) k_linbnd3d(double *f, int pb0, int pb1, int pb2, int pb3, int pb4,
                                                         int pb5, int pf, int all, int Nx, int Ny, int Nz,
                                                         const double *chr, double ex, int ne)
{
   const int tid = threadIdx.x, nthr = blockDim.x;
   const int phys_bdy[6] = {pb0, pb1, pb2, pb3, pb4, pb5};
   const int jlo = Ny < 2 ? Ny : 2, jhi = 1 > Ny - 1 ? 1 : Ny - 1;
   const int klo = Nz < 2 ? Nz : 2, khi = 1 > Nz - 1 ? 1 : Nz - 1;
#define F(i, j, k) f[((i)-1) + (long)Nx * (((j)-1) + (long)Ny * ((k)-1))]
#define X(i, j, k) (chr[((i)-1) + (long)Nx * (((j)-1) + (long)Ny * ((k)-1))] != ex)
#define PB(n) (phys_bdy[(n)-1] == pf || all)
#define FOR1(a, lo, hi) for (int a = (lo) + tid; a <= (hi); a += nthr)
#define FOR2(a, alo, ahi, b, blo, bhi)                                                                 \
   for (long q_ = tid, nb_ = (bhi) - (blo) + 1, n_ = ((ahi) - (alo) + 1) * nb_; nb_ > 0 && q_ < n_; \
        q_ += nthr)                                                                                   \
      for (int a = (alo) + (int)(q_ / nb_), b = (blo) + (int)(q_ % nb_), once_ = 1; once_; once_ = 0)
#define ONE if (tid == 0)
   if (PB(1)) {
      FOR2(j, jlo, jhi, k, klo, khi)
            if (ne || (X(3, j, k) && X(1, j, k))) F(2, j, k) = 0.5 * (F(3, j, k) + F(1, j, k));
   __syncthreads();
      if (Ny > 1 && PB(3))
         FOR1(k, klo, khi)
            if (ne || (X(3, 3, k) && X(3, 1, k) && X(1, 3, k) && X(1, 1, k)))
               F(2, 2, k) = 0.25 * (F(3, 3, k) + F(1, 3, k) + F(3, 1, k) + F(1, 1, k));
   __syncthreads();
      if (Ny > 1 && PB(4))
         FOR1(k, klo, khi)
            if (ne || (X(3, Ny - 2, k) && X(1, Ny - 2, k) && X(3, Ny, k) && X(1, Ny, k)))
               F(2, Ny - 1, k) = 0.25 * (F(3, Ny - 2, k) + F(1, Ny - 2, k) + F(3, Ny, k) + F(1, Ny, k));
   __syncthreads();
      if (Nz > 1 && PB(5))
         FOR1(j, 2, Ny - 1)
            if (ne || (X(3, j, 3) && X(1, j, 3) && X(3, j, 1) && X(1, j, 1)))
               F(2, j, 2) = 0.25 * (F(3, j, 3) + F(1, j, 3) + F(3, j, 1) + F(1, j, 1));
   __syncthreads();
      if (Nz > 1 && PB(6))
         FOR1(j, 2, Ny - 1)
            if (ne || (X(3, j, Nz - 2) && X(1, j, Nz - 2) && X(3, j, Nz) && X(1, j, Nz)))
               F(2, j, Nz - 1) = 0.25 * (F(3, j, Nz - 2) + F(1, j, Nz - 2) + F(3, j, Nz) + F(1, j, Nz));
   __syncthreads();
      ONE if (Nz > 1 && ((phys_bdy[2] == pf && phys_bdy[4] == pf) ||
                     (all && (ne || (X(3, 3, 3) && X(1, 3, 3) && X(3, 1, 3) && X(3, 3, 1) && X(1, 1, 3) &&
                                     X(1, 3, 1) && X(3, 1, 1) && X(1, 1, 1))))))
         F(2, 2, 2) = 0.125 * (F(3, 3, 3) + F(1, 3, 3) + F(3, 1, 3) + F(3, 3, 1) + F(1, 1, 3) + F(1, 3, 1) +
                               F(3, 1, 1) + F(1, 1, 1));
   __syncthreads();
      ONE if (Nz > 1 && ((phys_bdy[3] == pf && phys_bdy[4] == pf) ||
                     (all && (ne || (X(3, Ny - 2, 3) && X(1, Ny - 2, 3) && X(3, Ny, 3) && X(3, Ny - 2, 1) &&
                                     X(1, Ny, 3) && X(1, Ny - 2, 1) && X(3, Ny, 1) && X(1, Ny, 1))))))
         F(2, Ny - 1, 2) = 0.125 * (F(3, Ny - 2, 3) + F(1, Ny - 2, 3) + F(3, Ny, 3) + F(3, Ny - 2, 1) +
                                    F(1, Ny, 3) + F(1, Ny - 2, 1) + F(3, Ny, 1) + F(1, Ny, 1));
   __syncthreads();
      ONE if (Nz > 1 && ((phys_bdy[2] == pf && phys_bdy[5] == pf) ||
                     (all && (ne || (X(3, 3, Nz - 2) && X(1, 3, Nz - 2) && X(3, 1, Nz - 2) && X(3, 3, Nz) &&
                                     X(1, 1, Nz - 2) && X(1, 3, Nz) && X(3, 1, Nz) && X(1, 1, Nz))))))
         F(2, 2, Nz - 1) = 0.125 * (F(3, 3, Nz - 2) + F(1, 3, Nz - 2) + F(3, 1, Nz - 2) + F(3, 3, Nz) +
                                    F(1, 1, Nz - 2) + F(1, 3, Nz) + F(3, 1, Nz) + F(1, 1, Nz));
   __syncthreads();
      ONE if (Nz > 1 && ((phys_bdy[3] == pf && phys_bdy[5] == pf) ||
                     (all && (ne || (X(3, Ny - 2, Nz - 2) && X(1, Ny - 2, Nz - 2) && X(3, Ny, Nz - 2) &&
                                     X(3, Ny - 2, Nz) && X(1, Ny, Nz - 2) && X(1, Ny - 2, Nz) && X(3, Ny, Nz) &&
                                     X(1, Ny, Nz))))))
         F(2, Ny - 1, Nz - 1) = 0.125 * (F(3, Ny - 2, Nz - 2) + F(1, Ny - 2, Nz - 2) + F(3, Ny, Nz - 2) +
                                         F(3, Ny - 2, Nz) + F(1, Ny, Nz - 2) + F(1, Ny - 2, Nz) + F(3, Ny, Nz) +
                                         F(1, Ny, Nz));
   __syncthreads();
   }

   if (PB(2)) {
      FOR2(j, jlo, jhi, k, klo, khi)
            if (ne || (X(Nx - 2, j, k) && X(Nx, j, k))) F(Nx - 1, j, k) = 0.5 * (F(Nx - 2, j, k) + F(Nx, j, k));
   __syncthreads();
      if (Ny > 1 && PB(3))
         FOR1(k, klo, khi)
            if (ne || (X(Nx - 2, 3, k) && X(Nx, 3, k) && X(Nx - 2, 1, k) && X(Nx, 1, k)))
               F(Nx - 1, 2, k) = 0.25 * (F(Nx - 2, 3, k) + F(Nx, 3, k) + F(Nx - 2, 1, k) + F(Nx, 1, k));
   __syncthreads();
      if (Ny > 1 && PB(4))
         FOR1(k, klo, khi)
            if (ne || (X(Nx - 2, Ny - 2, k) && X(Nx, Ny - 2, k) && X(Nx - 2, Ny, k) && X(Nx, Ny, k)))
               F(Nx - 1, Ny - 1, k) =
                   0.25 * (F(Nx - 2, Ny - 2, k) + F(Nx, Ny - 2, k) + F(Nx - 2, Ny, k) + F(Nx, Ny, k));
   __syncthreads();
      if (Nz > 1 && PB(5))
         FOR1(j, 2, Ny - 1)
            if (ne || (X(Nx - 2, j, 3) && X(Nx, j, 3) && X(Nx - 2, j, 1) && X(Nx, j, 1)))
               F(Nx - 1, j, 2) = 0.25 * (F(Nx - 2, j, 3) + F(Nx, j, 3) + F(Nx - 2, j, 1) + F(Nx, j, 1));
   __syncthreads();
      if (Nz > 1 && PB(6))
         FOR1(j, 2, Ny - 1)
            if (ne || (X(Nx - 2, j, Nz - 2) && X(Nx, j, Nz - 2) && X(Nx - 2, j, Nz) && X(Nx, j, Nz)))
               F(Nx - 1, j, Nz - 1) =
                   0.25 * (F(Nx - 2, j, Nz - 2) + F(Nx, j, Nz - 2) + F(Nx - 2, j, Nz) + F(Nx, j, Nz));
   __syncthreads();
      ONE if (Nz > 1 && ((phys_bdy[2] == pf && phys_bdy[4] == pf) ||
                     (all && (ne || (X(Nx - 2, 3, 3) && X(Nx, 3, 3) && X(Nx - 2, 1, 3) && X(Nx - 2, 3, 1) &&
                                     X(Nx, 1, 3) && X(Nx, 3, 1) && X(Nx - 2, 1, 1) && X(Nx, 1, 1))))))
         F(Nx - 1, 2, 2) = 0.125 * (F(Nx - 2, 3, 3) + F(Nx, 3, 3) + F(Nx - 2, 1, 3) + F(Nx - 2, 3, 1) +
                                    F(Nx, 1, 3) + F(Nx, 3, 1) + F(Nx - 2, 1, 1) + F(Nx, 1, 1));
   __syncthreads();
      ONE if (Nz > 1 && ((phys_bdy[3] == pf && phys_bdy[4] == pf) ||
                     (all && (ne || (X(Nx - 2, Ny - 2, 3) && X(Nx, Ny - 2, 3) && X(Nx - 2, Ny, 3) &&
                                     X(Nx - 2, Ny - 2, 1) && X(Nx, Ny, 3) && X(Nx, Ny - 2, 1) &&
                                     X(Nx - 2, Ny, 1) && X(Nx, Ny, 1))))))
         F(Nx - 1, Ny - 1, 2) = 0.125 * (F(Nx - 2, Ny - 2, 3) + F(Nx, Ny - 2, 3) + F(Nx - 2, Ny, 3) +
                                         F(Nx - 2, Ny - 2, 1) + F(Nx, Ny, 3) + F(Nx, Ny - 2, 1) +
                                         F(Nx - 2, Ny, 1) + F(Nx, Ny, 1));
   __syncthreads();
      ONE if (Nz > 1 && ((phys_bdy[2] == pf && phys_bdy[5] == pf) ||
                     (all && (ne || (X(Nx - 2, 3, Nz - 2) && X(Nx, 3, Nz - 2) && X(Nx - 2, 1, Nz - 2) &&
                                     X(Nx - 2, 3, Nz) && X(Nx, 1, Nz - 2) && X(Nx, 3, Nz) && X(Nx - 2, 1, Nz) &&
                                     X(Nx, 1, Nz))))))
         F(Nx - 1, 2, Nz - 1) = 0.125 * (F(Nx - 2, 3, Nz - 2) + F(Nx, 3, Nz - 2) + F(Nx - 2, 1, Nz - 2) +
                                         F(Nx - 2, 3, Nz) + F(Nx, 1, Nz - 2) + F(Nx, 3, Nz) + F(Nx - 2, 1, Nz) +
                                         F(Nx, 1, Nz));
   __syncthreads();
      ONE if (Nz > 1 && ((phys_bdy[3] == pf && phys_bdy[5] == pf) ||
                     (all && (ne || (X(Nx - 2, Ny - 2, Nz - 2) && X(Nx, Ny, Nz) && X(Nx, Ny - 2, Nz - 2) &&
                                     X(Nx - 2, Ny, Nz - 2) && X(Nx - 2, Ny - 2, Nz) && X(Nx, Ny, Nz - 2) &&
                                     X(Nx, Ny - 2, Nz) && X(Nx - 2, Ny, Nz))))))
         F(Nx - 1, Ny - 1, Nz - 1) = 0.125 * (F(Nx - 2, Ny - 2, Nz - 2) + F(Nx, Ny, Nz) + F(Nx, Ny - 2, Nz - 2) +
                                              F(Nx - 2, Ny, Nz - 2) + F(Nx - 2, Ny - 2, Nz) + F(Nx, Ny, Nz - 2) +
                                              F(Nx, Ny - 2, Nz) + F(Nx - 2, Ny, Nz));
   __syncthreads();
   }

   if (Ny > 1 && PB(3)) {
      FOR2(i, 3, Nx - 2, k, klo, khi)
            if (ne || (X(i, 3, k) && X(i, 1, k))) F(i, 2, k) = 0.5 * (F(i, 3, k) + F(i, 1, k));
   __syncthreads();
      if (Nz > 1 && PB(5))
         FOR1(i, 3, Nx - 2)
            if (ne || (X(i, 3, 3) && X(i, 1, 3) && X(i, 3, 1) && X(i, 1, 1)))
               F(i, 2, 2) = 0.25 * (F(i, 3, 3) + F(i, 1, 3) + F(i, 3, 1) + F(i, 1, 1));
   __syncthreads();
      if (Nz > 1 && PB(6))
         FOR1(i, 3, Nx - 2)
            if (ne || (X(i, 3, Nz - 2) && X(i, 1, Nz - 2) && X(i, 3, Nz) && X(i, 1, Nz)))
               F(i, 2, Nz - 1) = 0.25 * (F(i, 3, Nz - 2) + F(i, 1, Nz - 2) + F(i, 3, Nz) + F(i, 1, Nz));
   __syncthreads();
   }

   if (Ny > 1 && PB(4)) {
      FOR2(i, 3, Nx - 2, k, klo, khi)
            if (ne || (X(i, Ny - 2, k) && X(i, Ny, k))) F(i, Ny - 1, k) = 0.5 * (F(i, Ny - 2, k) + F(i, Ny, k));
   __syncthreads();
      if (Nz > 1 && PB(5))
         FOR1(i, 3, Nx - 2)
            if (ne || (X(i, Ny - 2, 3) && X(i, Ny, 3) && X(i, Ny - 2, 1) && X(i, Ny, 1)))
               F(i, Ny - 1, 2) = 0.25 * (F(i, Ny - 2, 3) + F(i, Ny, 3) + F(i, Ny - 2, 1) + F(i, Ny, 1));
   __syncthreads();
      if (Nz > 1 && PB(6))
         FOR1(i, 3, Nx - 2)
            if (ne || (X(i, Ny - 2, Nz - 2) && X(i, Ny, Nz - 2) && X(i, Ny - 2, Nz) && X(i, Ny, Nz)))
               F(i, Ny - 1, Nz - 1) =
                   0.25 * (F(i, Ny - 2, Nz - 2) + F(i, Ny, Nz - 2) + F(i, Ny - 2, Nz) + F(i, Ny, Nz));
   __syncthreads();
   }

   if (Nz > 1 && PB(5))
      FOR2(i, 3, Nx - 2, j, 3, Ny - 2)
            if (ne || (X(i, j, 3) && X(i, j, 1))) F(i, j, 2) = 0.5 * (F(i, j, 3) + F(i, j, 1));
   __syncthreads();

   if (Nz > 1 && PB(6))
      FOR2(i, 3, Nx - 2, j, 3, Ny - 2)
            if (ne || (X(i, j, Nz - 2) && X(i, j, Nz))) F(i, j, Nz - 1) = 0.5 * (F(i, j, Nz - 2) + F(i, j, Nz));
   __syncthreads();
#undef F
#undef X
#undef PB
#undef FOR1
#undef FOR2
#undef ONE
}

extern "C" int pgb_linbnd3d(double *f, const int *phys_bdy, int which_bnd, int Nx, int Ny, int Nz, const double *chr,
                            double ex, int do_ex, void *stream)
{
   int pf = -1, all = 0;
   /* the Fortran stops on the first three; with Ny = 1 and Nz > 1 its corner
    * statements index j = Ny-2 < 1, outside f: refused */
   if (Nx < 3 || Ny == 2 || Nz == 2 || (Ny == 1 && Nz > 1))
      return fail_lb("pgb_linbnd3d: invalid grid dimension", 3);
   if (which_bnd == 3)
      all = 1;
   else if (which_bnd == 1)
      pf = 1;
   else if (which_bnd == 2)
      pf = 0;
   else
      return fail_lb("pgb_linbnd3d: which_bnd must be 1, 2 or 3", 3);
   if (do_ex != 0 && !chr) return fail_lb("pgb_linbnd3d: do_ex needs chr", 3);
   k_linbnd3d<<<1, LB_THREADS, 0, (cudaStream_t)stream>>>(f, phys_bdy[0], phys_bdy[1], phys_bdy[2], phys_bdy[3],
                                                           phys_bdy[4], phys_bdy[5], pf, all, Nx, Ny, Nz,
                                                           do_ex ? chr : f, ex, do_ex == 0);
   g_launches_lb++;
   cudaError_t e = cudaGetLastError();
   if (e != cudaSuccess) {
      snprintf(g_err_lb, sizeof(g_err_lb), "pgb_linbnd3d: %s", cudaGetErrorString(e));
      pgb_note_error(g_err_lb);
      return 11;
   }
   return 0;
}
