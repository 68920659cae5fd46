/*
 * Learned initial guess of libpamr_gb300: BF16 tensor-core 3x3x3
 * convolutions (tcgen05.mma, FP32 accumulation in tensor memory) and the
 * other kernels of a 4-level convolutional encoder-decoder that maps a
 * source rho to a guess of the solution u, with its training step (forward,
 * backward, Adam) on the GPU. The data layout is described in pgb_net.h.
 *
 * Convolution as an implicit GEMM: one CTA computes a tile of 128
 * consecutive padded voxels (M = 128) for all output channels (N = Cout),
 * K = 27 taps x Cin in steps of 16 channels. For each of the three z-taps
 * the CTA bulk-copies, per y-tap and channel block, the run of 130 voxels
 * the three x-taps read (x-taps are offsets of 16 bytes into it), plus the
 * weights of those nine taps, waits on an mbarrier, and one thread issues
 * the 9*Cin/16 MMAs. Operands are K-major without swizzle: a core matrix is
 * 8 voxels (rows) x 8 channels (16 bytes); SBO = 128 bytes between
 * consecutive 8-voxel groups, LBO = the distance between the two channel
 * blocks of a 16-channel step. The epilogue reads the accumulator with
 * tcgen05.ld (one voxel per thread), adds the bias, applies the activation, writes
 * BF16 and re-zeroes the padding.
 */
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include "pgb_dev.h"
#include "pgb_net.h"

static __thread char g_err_net[256];
static unsigned long long g_launches_net = 0;

extern "C" unsigned long long pgb_dev_launches_net(void) { return g_launches_net; }

static int check_net(const char *what)
{
   g_launches_net++;
   cudaError_t e = cudaGetLastError();
   if (e != cudaSuccess) {
      snprintf(g_err_net, sizeof(g_err_net), "%s: %s", what, cudaGetErrorString(e));
      pgb_note_error(g_err_net);
      return 1;
   }
   return 0;
}

static int arg_err(const char *msg)
{
   snprintf(g_err_net, sizeof(g_err_net), "%s", msg);
   pgb_note_error(g_err_net);
   return 12;
}

/* ------------------------------------------------------------ PTX pieces -- */
__device__ __forceinline__ uint32_t s_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t global_ns()
{
   uint64_t t;
   asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
   return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
   asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(s_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init()
{
   asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
   asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(s_addr(bar)), "r"(bytes)
                : "memory");
}

__device__ __forceinline__ bool mbar_try(uint64_t *bar, uint32_t phase)
{
   uint32_t ok;
   asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                " selp.u32 %0, 1, 0, p;\n}\n"
                : "=r"(ok)
                : "r"(s_addr(bar)), "r"(phase)
                : "memory");
   return ok != 0;
}

/* waits for the phase with a limit of about one second; false on timeout */
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t phase)
{
   const uint64_t t0 = global_ns();
   while (!mbar_try(bar, phase))
      if (global_ns() - t0 > 1000000000ull) return false;
   return true;
}

/* 1-D bulk copy global -> shared, completion counted on bar (16-byte
 * aligned addresses, size a multiple of 16) */
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
   asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
                   "r"(s_addr(dst)), "l"(src), "r"(bytes), "r"(s_addr(bar))
                : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols)
{
   asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(s_addr(dst)),
                "r"(ncols)
                : "memory");
   asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
   asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

/* D[tmem] (+)= A[smem] x B[smem], M x N x 16, BF16 in, FP32 accumulate */
__device__ __forceinline__ void mma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
   asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
                "l"(a), "l"(b), "r"(idesc), "r"(acc)
                : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar)
{
   asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(s_addr(bar))
                : "memory");
}

/* 32 lanes x 16 consecutive 32-bit columns: thread t gets lane (base + t) */
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v)
{
   uint32_t r[16];
   asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                  "=r"(r[15])
                : "r"(taddr));
   asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
   for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

/* shared-memory matrix descriptor, no swizzle (layout type 0), version 1 */
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
   return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
          ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

/* instruction descriptor, kind::f16: FP32 D, BF16 A and B, both K-major */
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N)
{
   return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

/* ------------------------------------------------------------ geometry -- */
static pgb_lvgeom make_geom(int W, int H, int D)
{
   pgb_lvgeom g;
   g.W = W;
   g.H = H;
   g.D = D;
   g.Wp = W + 2;
   g.Hp = H + 2;
   g.Dp = D + 2;
   g.plane = (long)g.Wp * g.Hp;
   g.margin = g.plane + g.Wp + 2 + 128;
   g.vtot = 2 * g.margin + g.plane * g.Dp;
   g.p0 = g.plane;
   g.ntile = (int)((D * g.plane + 127) / 128);
   return g;
}

/* the activation after every convolution but the last: leaky ReLU with
 * negative slope 1/8 (a power of two: scaling commutes with it and with
 * every rounding, so a bias-free net stays exactly homogeneous) */
#define LEAK 0.125f
__device__ __forceinline__ float leaky(float a) { return a > 0.f ? a : LEAK * a; }

/* ------------------------------------------------- tensor-core 3x3x3 conv -- */
#define CONV_RUN 130   /* voxels of one y/z-tap run (x-taps -1, 0, +1 of 128 outputs) */

template <int CIN, int COUT>
struct ConvSmem {
   static constexpr int KS = CIN / 16;                        /* 16-channel K steps per tap */
   static constexpr int A_BYTES = 3 * (CIN / 8) * CONV_RUN * 16;
   static constexpr int W_BYTES = 9 * CIN * COUT * 2;         /* nine taps of one z-tap */
   static constexpr int LOAD_BYTES = A_BYTES + W_BYTES;      /* bulk-copied per z-tap */
   /* 40 KB beyond the operands: every shared-memory address an MMA could
    * form from these descriptors stays inside the allocation */
   static constexpr int BYTES = LOAD_BYTES + 40 * 1024;
   static constexpr int NCOL = COUT < 32 ? 32 : COUT;         /* TMEM columns (power of 2) */
};

/* Weight image (global, BF16): for z-tap dz, the nine (dy,dx) taps, K steps
 * ks, half h, output channel co, 8 input channels:
 *   wimg[dz][dy*3+dx][ks][h][co][8] = w[tap][16ks + 8h + e][co] */
template <int CIN, int COUT>
__global__ void __launch_bounds__(128) k_conv_tc(const __nv_bfloat16 *in, __nv_bfloat16 *out,
                                                 const __nv_bfloat16 *wimg, const float *bias,
                                                 pgb_lvgeom g, int relu, int *err)
{
   typedef ConvSmem<CIN, COUT> S;
   extern __shared__ __align__(128) uint8_t smem[];
   uint8_t *sA = smem, *sW = smem + S::A_BYTES;
   __shared__ __align__(8) uint64_t bar_load, bar_mma;
   __shared__ uint32_t tmem_base;
   __shared__ int s_fail;
   const int tid = threadIdx.x, warp = tid >> 5;
   const long T = g.p0 + 128L * blockIdx.x;

   if (warp == 0) tmem_alloc(&tmem_base, S::NCOL);
   if (tid == 0) {
      mbar_init(&bar_load, 1);
      mbar_init(&bar_mma, 1);
      mbar_fence_init();
      s_fail = 0;
   }
   tc_fence_before();
   __syncthreads();
   tc_fence_after();
   const uint32_t taddr = tmem_base;
   constexpr uint32_t IDESC = idesc_bf16(128, COUT);

   for (int dz = 0; dz < 3; dz++) {
      if (tid == 0) {
         mbar_expect_tx(&bar_load, S::LOAD_BYTES);
         for (int dy = 0; dy < 3; dy++)
            for (int cb = 0; cb < CIN / 8; cb++) {
               const long v = g.margin + T + (dz - 1) * g.plane + (dy - 1) * (long)g.Wp - 1;
               bulk_g2s(sA + (dy * (CIN / 8) + cb) * CONV_RUN * 16, in + ((long)cb * g.vtot + v) * 8,
                        CONV_RUN * 16, &bar_load);
            }
         bulk_g2s(sW, wimg + (long)dz * (S::W_BYTES / 2), S::W_BYTES, &bar_load);
      }
      if (!mbar_wait(&bar_load, dz & 1)) s_fail = 1;
      __syncthreads();
      if (s_fail) break;
      if (tid == 0) {
         tc_fence_after();
         for (int dy = 0; dy < 3; dy++)
            for (int dx = 0; dx < 3; dx++)
               for (int ks = 0; ks < S::KS; ks++) {
                  const uint32_t a = s_addr(sA) + ((dy * (CIN / 8) + 2 * ks) * CONV_RUN + dx) * 16;
                  const uint32_t b = s_addr(sW) + (((dy * 3 + dx) * S::KS + ks) * 2 * COUT) * 16;
                  mma_bf16(taddr, sdesc(a, CONV_RUN * 16, 128), sdesc(b, COUT * 16, 128), IDESC,
                           (dz | dy | dx | ks) != 0);
               }
         mma_commit(&bar_mma);
      }
      if (!mbar_wait(&bar_mma, dz & 1)) s_fail = 1;
      __syncthreads();
      if (s_fail) break;
   }

   if (!s_fail) {
      tc_fence_after();
      const long P = T + tid;   /* this thread's voxel (TMEM lane tid) */
      const long x = P % g.Wp, y = (P / g.Wp) % g.Hp, z = P / g.plane;
      const bool pad = x == 0 || x == g.Wp - 1 || y == 0 || y == g.Hp - 1 || z == 0 || z >= g.Dp - 1;
      const uint32_t tw = taddr + ((uint32_t)(warp * 32) << 16);
#pragma unroll
      for (int c16 = 0; c16 < COUT / 16; c16++) {
         float v[16];
         tmem_ld16(tw + c16 * 16, v);
#pragma unroll
         for (int h = 0; h < 2; h++) {
            uint32_t pk[4];
#pragma unroll
            for (int e = 0; e < 4; e++) {
               float a0 = v[h * 8 + 2 * e], a1 = v[h * 8 + 2 * e + 1];
               if (bias) {
                  a0 += bias[c16 * 16 + h * 8 + 2 * e];
                  a1 += bias[c16 * 16 + h * 8 + 2 * e + 1];
               }
               if (relu) {
                  a0 = leaky(a0);
                  a1 = leaky(a1);
               }
               if (pad) a0 = a1 = 0.f;
               __nv_bfloat162 b2 = __floats2bfloat162_rn(a0, a1);
               pk[e] = *reinterpret_cast<uint32_t *>(&b2);
            }
            const long cb = c16 * 2 + h;
            *reinterpret_cast<uint4 *>(out + (cb * g.vtot + g.margin + P) * 8) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
         }
      }
   } else {
      /* a wait ran out: give the copies and MMAs in flight another bounded
       * chance to land before the shared and tensor memory are released */
      mbar_wait(&bar_load, 0);
      mbar_wait(&bar_mma, 0);
      if (tid == 0 && err) atomicExch(err, 1);
   }
   tc_fence_before();
   __syncthreads();
   if (warp == 0) tmem_dealloc(taddr, S::NCOL);
}

template <int CIN, int COUT>
static int launch_conv(const void *in, void *out, const void *wimg, const float *bias, const pgb_lvgeom &g,
                       int relu, int *err, cudaStream_t st)
{
   typedef ConvSmem<CIN, COUT> S;
   static bool attr = false;
   if (!attr) {
      if (cudaFuncSetAttribute(k_conv_tc<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, S::BYTES) !=
          cudaSuccess)
         return check_net("conv attribute");
      attr = true;
   }
   k_conv_tc<CIN, COUT><<<g.ntile, 128, S::BYTES, st>>>((const __nv_bfloat16 *)in, (__nv_bfloat16 *)out,
                                                         (const __nv_bfloat16 *)wimg, bias, g, relu, err);
   return check_net("conv_tc") ? 11 : 0;
}

/* ------------------------------------- tensor-core 3x3x3 conv, z-marching -- */
/* The same convolution for 16/32-channel layers, persistent and pipelined.
 * Tiles are 128 consecutive padded voxels of one plane (tile j of plane z
 * starts at p0 + z plane + 128 j; the last tile of a plane is cut at the
 * plane's end). A work unit is one tile column j over a chunk of planes;
 * the CTA marches it in z. The operands of one input plane (three runs of
 * 130 voxels per channel block, y-taps -1..1) are one pipeline stage,
 * bulk-copied once and used by the three output planes that read it
 * (z-taps), so each plane's runs cross L2 -> shared memory once per unit
 * instead of three times. Roles: warp 0 lane 0 streams stages into a
 * ring of NST stages (full/empty mbarriers); warp 1 lane 0 issues the 27 x CIN/16
 * MMAs of a tile into one of two TMEM accumulators (commits free the
 * input stage the next tile no longer reads, and hand the accumulator to
 * the epilogue); warps 2-5 read an accumulator (tcgen05.ld, one voxel per
 * thread), add the bias, apply the activation, zero padding voxels, store
 * BF16, and hand the accumulator back. The layer's weights stay in shared
 * memory for the whole kernel. Every wait is bounded; on a timeout the
 * roles stop, the error flag is set and TMEM is freed. */
#define CZ_THREADS 192

template <int CIN, int COUT>
struct ConvZSmem {
   /* a tile reads three stages; the rest stream in behind them. 16-channel
    * inputs keep a shorter ring so that three CTAs (three MMA issuers)
    * share an SM */
   static constexpr int NST = CIN == 16 ? 4 : 6;
   static constexpr int KS = CIN / 16;
   static constexpr int STAGE = 3 * (CIN / 8) * CONV_RUN * 16;   /* one input plane's runs */
   static constexpr int W_ALL = 27 * CIN * COUT * 2;             /* all taps, packed image */
   /* no slack: the highest byte an A descriptor reaches (last run block,
    * x-tap +1, second K half, row group 15) is the last byte of its stage,
    * and a B descriptor stays inside its tap's 2 x COUT x 16 bytes */
   static constexpr int BYTES = W_ALL + NST * STAGE;
   static constexpr int NCOL = COUT < 32 ? 32 : COUT;            /* columns of one accumulator */
};

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
   asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(s_addr(bar)) : "memory");
}

template <int CIN, int COUT>
__global__ void __launch_bounds__(CZ_THREADS) k_conv_tcz(const __nv_bfloat16 *in, __nv_bfloat16 *out,
                                                         const __nv_bfloat16 *wimg, const float *bias, pgb_lvgeom g,
                                                         int relu, int jt, int zc, int nunit, int *err)
{
   typedef ConvZSmem<CIN, COUT> S;
   extern __shared__ __align__(128) uint8_t smem[];
   uint8_t *sW = smem, *sA = smem + S::W_ALL;
   __shared__ __align__(8) uint64_t full[S::NST], empty[S::NST], tfull[2], tempty[2], wbar;
   __shared__ uint32_t tmem_base;
   __shared__ int s_fail_;
   volatile int &s_fail = s_fail_;
   const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

   if (warp == 0) tmem_alloc(&tmem_base, 2 * S::NCOL);
   if (tid == 0) {
      for (int s = 0; s < S::NST; s++) {
         mbar_init(&full[s], 1);
         mbar_init(&empty[s], 1);
      }
      for (int b = 0; b < 2; b++) {
         mbar_init(&tfull[b], 1);
         mbar_init(&tempty[b], 4);
      }
      mbar_init(&wbar, 1);
      mbar_fence_init();
      s_fail = 0;
   }
   tc_fence_before();
   __syncthreads();
   tc_fence_after();
   const uint32_t taddr = tmem_base;
   constexpr uint32_t IDESC = idesc_bf16(128, COUT);

   if (warp == 0) {
      /* producer */
      if (lane == 0) {
         mbar_expect_tx(&wbar, S::W_ALL);
         bulk_g2s(sW, wimg, S::W_ALL, &wbar);
         uint32_t cnt = 0;
         for (int u = blockIdx.x; u < nunit && !s_fail; u += gridDim.x) {
            const int j = u % jt, z0 = (u / jt) * zc, z1 = min(g.D, z0 + zc);
            for (int zz = z0 - 1; zz <= z1 && !s_fail; zz++, cnt++) {
               const int s = cnt % S::NST;
               if (!mbar_wait(&empty[s], ((cnt / S::NST) & 1) ^ 1)) {
                  s_fail = 1;
                  break;
               }
               mbar_expect_tx(&full[s], S::STAGE);
               const long T = g.p0 + (long)zz * g.plane + 128L * j;
               for (int dy = 0; dy < 3; dy++)
                  for (int cb = 0; cb < CIN / 8; cb++) {
                     const long v = g.margin + T + (dy - 1) * (long)g.Wp - 1;
                     bulk_g2s(sA + s * S::STAGE + (dy * (CIN / 8) + cb) * CONV_RUN * 16,
                              in + ((long)cb * g.vtot + v) * 8, CONV_RUN * 16, &full[s]);
                  }
            }
         }
         /* tail: every stage handed out is released (its last MMAs done)
          * before the CTA exits, so no arrival lands after the memory is freed */
         for (uint32_t k = cnt > S::NST ? cnt - S::NST : 0; k < cnt && !s_fail; k++)
            if (!mbar_wait(&empty[k % S::NST], (k / S::NST) & 1)) s_fail = 1;
      }
   } else if (warp == 1) {
      /* MMA issuer */
      if (lane == 0) {
         bool ok = mbar_wait(&wbar, 0);
         uint32_t cnt = 0, tc = 0;
         const uint64_t a_desc0 = sdesc(s_addr(sA), CONV_RUN * 16, 128), b_desc0 = sdesc(s_addr(sW), COUT * 16, 128);
         for (int u = blockIdx.x; u < nunit && ok && !s_fail; u += gridDim.x) {
            const int z0 = (u / jt) * zc, z1 = min(g.D, z0 + zc);
            const uint32_t base = cnt;   /* stage sequence number of plane z0-1 */
            /* planes z0-1 and z0 */
            for (int q = 0; q < 2 && ok; q++)
               ok = mbar_wait(&full[(base + q) % S::NST], ((base + q) / S::NST) & 1);
            for (int z = z0; z < z1 && ok; z++, tc++) {
               const uint32_t nz = base + (z - z0) + 2;   /* plane z+1 */
               ok = mbar_wait(&full[nz % S::NST], (nz / S::NST) & 1) &&
                    mbar_wait(&tempty[tc & 1], ((tc >> 1) & 1) ^ 1);
               if (!ok) break;
               tc_fence_after();
               const uint32_t acc = taddr + (tc & 1) * S::NCOL;
#pragma unroll
               for (int dz = 0; dz < 3; dz++) {
                  const uint32_t st = (base + (z - z0) + dz) % S::NST;
                  /* descriptors are linear in the address (14-bit field of
                   * address / 16, no carry below 256 KB): one base each, plus
                   * compile-time offsets */
                  const uint64_t da = a_desc0 + ((st * S::STAGE) >> 4);
#pragma unroll
                  for (int dy = 0; dy < 3; dy++)
#pragma unroll
                     for (int dx = 0; dx < 3; dx++)
#pragma unroll
                        for (int ks = 0; ks < S::KS; ks++) {
                           const uint32_t ao = ((dy * (CIN / 8) + 2 * ks) * CONV_RUN + dx) * 16;
                           const uint32_t bo = ((((dz * 3 + dy) * 3 + dx) * S::KS + ks) * 2 * COUT) * 16;
                           mma_bf16(acc, da + (ao >> 4), b_desc0 + (bo >> 4), IDESC, (dz | dy | dx | ks) != 0);
                        }
               }
               mma_commit(&empty[(base + (z - z0)) % S::NST]);   /* plane z-1 is done */
               mma_commit(&tfull[tc & 1]);
            }
            if (ok) {   /* planes z1-1 and z1 are done too */
               mma_commit(&empty[(base + (z1 - z0)) % S::NST]);
               mma_commit(&empty[(base + (z1 - z0) + 1) % S::NST]);
               cnt = base + (z1 - z0) + 2;
            }
         }
         if (!ok) s_fail = 1;
      }
   } else {
      /* epilogue: warps 2..5 own TMEM lanes 32 (warp % 4) .. + 31 */
      const int row = 32 * (warp & 3) + lane;
      const int plane = (int)g.plane;
      float bv[COUT];
#pragma unroll
      for (int c = 0; c < COUT; c++) bv[c] = bias ? bias[c] : 0.f;
      uint32_t tc = 0;
      for (int u = blockIdx.x; u < nunit && !s_fail; u += gridDim.x) {
         const int j = u % jt, z0 = (u / jt) * zc, z1 = min(g.D, z0 + zc);
         for (int z = z0; z < z1; z++, tc++) {
            if (!mbar_wait(&tfull[tc & 1], (tc >> 1) & 1)) {
               s_fail = 1;
               break;
            }
            tc_fence_after();
            const int q = 128 * j + row;                                  /* offset in the plane */
            const long P = g.p0 + (long)z * g.plane + q;                  /* this thread's voxel */
            const bool mine = q < plane;                                  /* not the next plane's */
            const int y = q / g.Wp, x = q - y * g.Wp;
            const bool pad = x == 0 || x == g.Wp - 1 || y == 0 || y == g.Hp - 1;
            const uint32_t tw = taddr + (tc & 1) * S::NCOL + ((uint32_t)(32 * (warp & 3)) << 16);
#pragma unroll
            for (int c16 = 0; c16 < COUT / 16; c16++) {
               float v[16];
               tmem_ld16(tw + c16 * 16, v);
#pragma unroll
               for (int h = 0; h < 2; h++) {
                  uint32_t pk[4];
#pragma unroll
                  for (int e = 0; e < 4; e++) {
                     float a0 = v[h * 8 + 2 * e] + bv[c16 * 16 + h * 8 + 2 * e];
                     float a1 = v[h * 8 + 2 * e + 1] + bv[c16 * 16 + h * 8 + 2 * e + 1];
                     if (relu) {
                        a0 = leaky(a0);
                        a1 = leaky(a1);
                     }
                     if (pad) a0 = a1 = 0.f;
                     __nv_bfloat162 b2 = __floats2bfloat162_rn(a0, a1);
                     pk[e] = *reinterpret_cast<uint32_t *>(&b2);
                  }
                  if (mine) {
                     const long cb = c16 * 2 + h;
                     *reinterpret_cast<uint4 *>(out + (cb * g.vtot + g.margin + P) * 8) =
                         make_uint4(pk[0], pk[1], pk[2], pk[3]);
                  }
               }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&tempty[tc & 1]);
         }
         if (s_fail) break;
      }
   }
   __syncthreads();
   if (s_fail) {
      /* let copies and MMAs in flight land (about a millisecond) before the
       * shared and tensor memory are released */
      const uint64_t t0 = global_ns();
      while (global_ns() - t0 < 1000000ull) {
      }
      if (tid == 0 && err) atomicExch(err, 1);
   }
   tc_fence_before();
   __syncthreads();
   if (warp == 0) tmem_dealloc(taddr, 2 * S::NCOL);
}

/* an upper bound on the CTAs of the persistent convolution (0: one wave of
 * the whole GPU); a prediction running beside a solve leaves it the rest of
 * the SMs (pgb_net_set_grid_cap) */
static int g_tcz_cap = 0;

template <int CIN, int COUT>
static int launch_convz(const void *in, void *out, const void *wimg, const float *bias, const pgb_lvgeom &g,
                        int relu, int *err, cudaStream_t st)
{
   typedef ConvZSmem<CIN, COUT> S;
   static bool attr = false;
   if (!attr) {
      if (cudaFuncSetAttribute(k_conv_tcz<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, S::BYTES) !=
          cudaSuccess)
         return check_net("convz attribute");
      attr = true;
   }
   const int jt = (int)((g.plane + 127) / 128);
   const int per_sm = (227 * 1024) / (S::BYTES + 1024) > 0 ? (227 * 1024) / (S::BYTES + 1024) : 1;
   const int want = 2 * 152 * per_sm;
   int zc = 32;
   while (zc > 1 && (long)jt * ((g.D + zc - 1) / zc) < want) zc /= 2;
   const int nunit = jt * ((g.D + zc - 1) / zc);
   int grid = nunit < 152 * per_sm ? nunit : 152 * per_sm;
   if (g_tcz_cap > 0 && grid > g_tcz_cap) grid = g_tcz_cap;
   k_conv_tcz<CIN, COUT><<<grid, CZ_THREADS, S::BYTES, st>>>((const __nv_bfloat16 *)in, (__nv_bfloat16 *)out,
                                                             (const __nv_bfloat16 *)wimg, bias, g, relu, jt, zc,
                                                             nunit, err);
   return check_net("conv_tcz") ? 11 : 0;
}

#define CONV_CASE(a, b) \
   if (cin == a && cout == b) return launch_conv<a, b>(in, out, wimg, bias, g, relu, err, st);

#define CONVZ_CASE(a, b) \
   if (cin == a && cout == b) return launch_convz<a, b>(in, out, wimg, bias, g, relu, err, st);

static int conv_dispatch(int cin, int cout, const void *in, void *out, const void *wimg, const float *bias,
                         const pgb_lvgeom &g, int relu, int *err, cudaStream_t st)
{
   /* 16/32-channel layers: the z-marching pipelined kernel; 64-channel
    * layers (weights too large to keep resident beside the stages): one CTA
    * per tile */
   CONVZ_CASE(16, 16)
   CONVZ_CASE(16, 32)
   CONVZ_CASE(32, 16)
   CONVZ_CASE(32, 32)
   CONV_CASE(16, 16)
   CONV_CASE(16, 32)
   CONV_CASE(16, 64)
   CONV_CASE(32, 16)
   CONV_CASE(32, 32)
   CONV_CASE(32, 64)
   CONV_CASE(64, 16)
   CONV_CASE(64, 32)
   CONV_CASE(64, 64)
   return arg_err("conv3d: channel counts must be 16, 32 or 64");
}

/* w[27][cin][cout] FP32 (tap = dz*9 + dy*3 + dx) -> the kernel's BF16 image;
 * flip = 1 makes the image of the adjoint convolution (tap 26 - t, channels
 * swapped: the image then has cin' = cout, cout' = cin) */
__global__ void k_pack_weights(const float *w, __nv_bfloat16 *img, int cin, int cout, int flip)
{
   const int ci_n = flip ? cout : cin, co_n = flip ? cin : cout;   /* channels of the packed conv */
   const int ks_n = ci_n / 16;
   const long n = 27L * ci_n * co_n;
   for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < (int)n; q += gridDim.x * blockDim.x) {
      /* q enumerates the image: [dz][t9][ks][h][co][e] */
      const int e = (int)(q % 8);
      long r = q / 8;
      const int co = (int)(r % co_n);
      r /= co_n;
      const int h = (int)(r % 2);
      r /= 2;
      const int ks = (int)(r % ks_n);
      r /= ks_n;
      const int t9 = (int)(r % 9), dz = (int)(r / 9);
      const int tap = dz * 9 + t9, ci = 16 * ks + 8 * h + e;
      float v;
      if (flip) v = w[((long)(26 - tap) * cin + co) * cout + ci];   /* adjoint: w[26-t][co'][ci'] */
      else v = w[((long)tap * cin + ci) * cout + co];
      img[q] = __float2bfloat16_rn(v);
   }
}

extern "C" int pgb_conv3d_geometry(int W, int H, int D, long *vtot, long *margin)
{
   pgb_lvgeom g = make_geom(W, H, D);
   if (vtot) *vtot = g.vtot;
   if (margin) *margin = g.margin;
   return 0;
}

extern "C" int pgb_conv3d_pack_weights(const float *w, void *img, int cin, int cout, int adjoint, void *stream)
{
   if ((cin % 16) || (cout % 16)) return arg_err("pack_weights: channel counts must be multiples of 16");
   k_pack_weights<<<256, 256, 0, (cudaStream_t)stream>>>(w, (__nv_bfloat16 *)img, cin, cout, adjoint);
   return check_net("pack_weights") ? 11 : 0;
}

extern "C" int pgb_conv3d_bf16(const void *in, void *out, const void *wimg, const float *bias, int W, int H,
                               int D, int cin, int cout, int relu, int *err, void *stream)
{
   if (W < 1 || H < 1 || D < 1) return arg_err("conv3d: empty volume");
   pgb_lvgeom g = make_geom(W, H, D);
   return conv_dispatch(cin, cout, in, out, wimg, bias, g, relu, err, (cudaStream_t)stream);
}

/* ------------------------------------------- CUDA-core kernels of the net -- */
typedef __nv_bfloat16 bf16;

/* x, y, z of voxel q of the interior volume (x fastest), in 32-bit
 * arithmetic: volumes here stay below 2^31 voxels (pgb_net_create bounds n) */
__device__ __forceinline__ void xyz(int q, const pgb_lvgeom &g, int &x, int &y, int &z)
{
   const int wh = g.W * g.H;
   z = q / wh;
   const int r = q - z * wh;
   y = r / g.W;
   x = r - y * g.W;
}

__device__ __forceinline__ long vox(const pgb_lvgeom &g, int x, int y, int z)
{
   return g.margin + (x + 1) + (long)g.Wp * ((y + 1) + (long)g.Hp * (z + 1));
}

__device__ __forceinline__ void load8(const bf16 *a, long idx, float *v)
{
   const uint4 u = *reinterpret_cast<const uint4 *>(a + idx * 8);
   const __nv_bfloat162 *h = reinterpret_cast<const __nv_bfloat162 *>(&u);
#pragma unroll
   for (int e = 0; e < 4; e++) {
      float2 f = __bfloat1622float2(h[e]);
      v[2 * e] = f.x;
      v[2 * e + 1] = f.y;
   }
}

__device__ __forceinline__ void store8(bf16 *a, long idx, const float *v)
{
   uint32_t pk[4];
#pragma unroll
   for (int e = 0; e < 4; e++) {
      __nv_bfloat162 b2 = __floats2bfloat162_rn(v[2 * e], v[2 * e + 1]);
      pk[e] = *reinterpret_cast<uint32_t *>(&b2);
   }
   *reinterpret_cast<uint4 *>(a + idx * 8) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
}

/* first layer, 1 -> 16 channels: a0 = leaky(conv(s_in * rho) + b); rho is
 * the n^3 FP64 grid, the net sees its points 0..n-2 in each dimension
 * (zero beyond), read here through its FP32 copy r32 */
/* r32 = s_in * rho as FP32 in the level-0 padded layout (one channel,
 * zero on the padding and margins, which nothing writes), converted once
 * per voxel: the first layer and its weight gradient read each value 27
 * times, at fixed offsets without bounds tests */
__global__ void k_rho32(const double *rho, int n, float s_in, const double *q, float *r32, pgb_lvgeom g)
{
   const long nv = (long)g.W * g.H * g.D;
   if (q) s_in = (float)(1.0 / fmax(*q, 1e-300));   /* the source's charge, computed on the device */
   for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < (int)nv; q += gridDim.x * blockDim.x) {
      int x, y, z;
      xyz(q, g, x, y, z);
      r32[vox(g, x, y, z)] = s_in * (float)rho[x + (long)n * (y + (long)n * z)];
   }
}

__global__ void k_in_fwd(const float *r32, const float *w, const float *b, bf16 *out, pgb_lvgeom g)
{
   /* one voxel per thread: with a loop over voxels the compiler would keep
    * all 432 weights in registers across it */
   __shared__ float4 sw[27 * 4];   /* the weights, staged once per block */
   for (int i = threadIdx.x; i < 27 * 4; i += blockDim.x)
      sw[i] = make_float4(w[4 * i], w[4 * i + 1], w[4 * i + 2], w[4 * i + 3]);
   __syncthreads();
   const int q = blockIdx.x * blockDim.x + threadIdx.x;
   if (q >= g.W * g.H * g.D) return;
   int x, y, z;
   xyz(q, g, x, y, z);
   float acc[16];
#pragma unroll
   for (int c = 0; c < 16; c++) acc[c] = b[c];
   const long p0 = vox(g, x, y, z);
#pragma unroll 3
   for (int t = 0; t < 27; t++) {
      const float r = r32[p0 + (t / 9 - 1) * g.plane + ((t / 3) % 3 - 1) * (long)g.Wp + (t % 3 - 1)];
#pragma unroll
      for (int c4 = 0; c4 < 4; c4++) {
         const float4 wv = sw[t * 4 + c4];
         acc[4 * c4] = fmaf(r, wv.x, acc[4 * c4]);
         acc[4 * c4 + 1] = fmaf(r, wv.y, acc[4 * c4 + 1]);
         acc[4 * c4 + 2] = fmaf(r, wv.z, acc[4 * c4 + 2]);
         acc[4 * c4 + 3] = fmaf(r, wv.w, acc[4 * c4 + 3]);
      }
   }
#pragma unroll
   for (int c = 0; c < 16; c++) acc[c] = leaky(acc[c]);
   store8(out, p0, acc);
   store8(out, g.vtot + p0, acc + 8);
}

/* last layer, 16 -> 1 channel, no activation: up = conv(a) + b, as FP32 on
 * the net volume (x fastest) */
__global__ void k_out_fwd(const bf16 *a, const float *w, const float *b, float *up, pgb_lvgeom g)
{
   /* a thread computes four voxels along z: each 16-channel vector it loads
    * serves every output plane that reads it; each output still sums its
    * taps in tap order (z, then y, then x), as one voxel per thread would */
   __shared__ float4 sw[27 * 4];   /* the weights, staged once per block */
   for (int i = threadIdx.x; i < 27 * 4; i += blockDim.x)
      sw[i] = make_float4(w[4 * i], w[4 * i + 1], w[4 * i + 2], w[4 * i + 3]);
   __syncthreads();
   const int zb = (g.D + 3) / 4;
   const long nw = (long)g.W * g.H * zb;
   for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < (int)nw; q += gridDim.x * blockDim.x) {
      int x, y, z0;
      xyz(q, g, x, y, z0);
      z0 *= 4;
      const int nz = g.D - z0 < 4 ? g.D - z0 : 4;
      float acc[4];
#pragma unroll
      for (int k = 0; k < 4; k++) acc[k] = b[0];
      for (int zz = z0 - 1; zz <= z0 + nz; zz++)
#pragma unroll
         for (int t9 = 0; t9 < 9; t9++) {
            const long p = vox(g, x + t9 % 3 - 1, y + t9 / 3 - 1, zz);
            float v[16];
            load8(a, p, v);
            load8(a, g.vtot + p, v + 8);
#pragma unroll
            for (int k = 0; k < 4; k++) {
               const int dz = zz - (z0 + k) + 1;
               if (k >= nz || dz < 0 || dz > 2) continue;
               const float4 *wt = sw + (dz * 9 + t9) * 4;
#pragma unroll
               for (int c4 = 0; c4 < 4; c4++) {
                  const float4 wv = wt[c4];
                  acc[k] = fmaf(v[4 * c4], wv.x, acc[k]);
                  acc[k] = fmaf(v[4 * c4 + 1], wv.y, acc[k]);
                  acc[k] = fmaf(v[4 * c4 + 2], wv.z, acc[k]);
                  acc[k] = fmaf(v[4 * c4 + 3], wv.w, acc[k]);
               }
            }
         }
      for (int k = 0; k < nz; k++) up[x + (long)g.W * (y + (long)g.H * (z0 + k))] = acc[k];
   }
}

/* u (n^3 FP64) = s_out * up on points 1..n-2 of the net volume, 0 on the
 * grid's boundary points */
__global__ void k_out_store(const float *up, double *u, int n, double s_out, const double *q, double gain,
                            pgb_lvgeom g)
{
   if (q) s_out = gain * fmax(*q, 1e-300);
   const long nn = (long)n * n * n;
   for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < (int)nn; q += gridDim.x * blockDim.x) {
      const int z = q / (n * n), r = q - z * n * n, y = r / n, x = r - y * n;
      double v = 0.0;
      if (x > 0 && y > 0 && z > 0 && x < n - 1 && y < n - 1 && z < n - 1)
         v = s_out * (double)up[x + (long)g.W * (y + (long)g.H * z)];
      u[q] = v;
   }
}

/* Energy-norm scaling of a guess of lap u = rho (u = 0 on the boundary,
 * spacing h): with A = -lap (symmetric positive definite), the factor that
 * minimises |alpha u - u*|_A is alpha = <u, rho> / <u, lap u>. This kernel
 * accumulates the two sums over the interior points in FP64; k_scale_guess
 * applies alpha, or -- when the guess is not finite (a NaN or Inf anywhere
 * makes a sum so), is zero, or its alpha is outside [1/16, 16], which a
 * trained net's guess never needs -- replaces the guess by u = 0, the plain
 * solve's initial guess, and counts the rejection in dots[2]. */
__global__ void k_energy_dots(const double *rho, const double *u, int n, double inv_h2, double *dots)
{
   __shared__ double sm[2][8];
   const long nn = (long)n * n * n, s1 = n, s2 = (long)n * n;
   double a = 0, b = 0;
   for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < (int)nn; q += gridDim.x * blockDim.x) {
      const int z = q / (n * n), r = q - z * n * n, y = r / n, x = r - y * n;
      if (x == 0 || y == 0 || z == 0 || x == n - 1 || y == n - 1 || z == n - 1) continue;
      const double c = u[q];
      const double lap = (u[q - 1] + u[q + 1] + u[q - s1] + u[q + s1] + u[q - s2] + u[q + s2] - 6.0 * c) * inv_h2;
      a += c * rho[q];
      b += c * lap;
   }
   for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, o);
      b += __shfl_down_sync(0xffffffffu, b, o);
   }
   if ((threadIdx.x & 31) == 0) sm[0][threadIdx.x >> 5] = a, sm[1][threadIdx.x >> 5] = b;
   __syncthreads();
   if (threadIdx.x == 0) {
      double ta = 0, tb = 0;
      for (int i = 0; i < (int)(blockDim.x >> 5); i++) ta += sm[0][i], tb += sm[1][i];
      atomicAdd(&dots[0], ta);
      atomicAdd(&dots[1], tb);
   }
}

__global__ void k_scale_guess(double *u, long nn, double *dots)
{
   const double a = dots[0], b = dots[1];
   const double alpha = b != 0.0 ? a / b : 0.0;
   const bool ok = isfinite(a) && isfinite(b) && b != 0.0 && isfinite(alpha) && alpha >= 0.0625 && alpha <= 16.0;
   if (!ok && blockIdx.x == 0 && threadIdx.x == 0) dots[2] += 1.0;
   for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < (int)nn; q += gridDim.x * blockDim.x)
      u[q] = ok ? u[q] * alpha : 0.0;
}

/* MSE over points 1..n-2: loss += sum (up - ut/s_out)^2 / N, gup = dloss/dup */
__global__ void k_loss(const float *up, const float *ut, int n, float inv_s_out, float *gup, double *loss,
                       pgb_lvgeom g)
{
   __shared__ double sm[8];
   const long nv = (long)g.W * g.H * g.D;
   const double inv_n = 1.0 / ((double)(n - 2) * (n - 2) * (n - 2));
   double acc = 0;
   for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < (int)nv; q += gridDim.x * blockDim.x) {
      int x, y, z;
      xyz(q, g, x, y, z);
      float gr = 0.f;
      if (x > 0 && y > 0 && z > 0) {
         const float d = up[q] - inv_s_out * ut[x + (long)n * (y + (long)n * z)];
         acc += (double)d * d;
         gr = (float)(2.0 * inv_n) * d;
      }
      gup[q] = gr;
   }
   for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
   if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
   __syncthreads();
   if (threadIdx.x == 0) {
      double s = 0;
      for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += sm[i];
      atomicAdd(loss, s * inv_n);
   }
}

/* last layer backward-data: ga (16 ch, BF16 layout) = adjoint conv of gup */
__global__ void k_out_bwd_data(const float *gup, const float *w, bf16 *ga, pgb_lvgeom g)
{
   const long nv = (long)g.W * g.H * g.D;
   for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < (int)nv; q += gridDim.x * blockDim.x) {
      int x, y, z;
      xyz(q, g, x, y, z);
      float acc[16];
#pragma unroll
      for (int c = 0; c < 16; c++) acc[c] = 0.f;
      for (int t = 0; t < 27; t++) {   /* the output voxel v - off(t) reads this voxel with tap t */
         const int xx = x - (t % 3 - 1), yy = y - ((t / 3) % 3 - 1), zz = z - (t / 9 - 1);
         if (xx < 0 || yy < 0 || zz < 0 || xx >= g.W || yy >= g.H || zz >= g.D) continue;
         const float gv = gup[xx + (long)g.W * (yy + (long)g.H * zz)];
#pragma unroll
         for (int c = 0; c < 16; c++) acc[c] = fmaf(gv, w[t * 16 + c], acc[c]);
      }
      const long p = vox(g, x, y, z);
      store8(ga, p, acc);
      store8(ga, g.vtot + p, acc + 8);
   }
}

__device__ void block_add(float v, float *red, float *dst)
{
   red[threadIdx.x] = v;
   __syncthreads();
   for (int k = blockDim.x / 2; k > 0; k >>= 1) {
      if ((int)threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
      __syncthreads();
   }
   if (threadIdx.x == 0 && dst) atomicAdd(dst, red[0]);
   __syncthreads();
}

/* last layer dW: dw[t][c] += sum_v a[v + off t][c] gup[v] (cin = 16), db */
__global__ void k_out_bwd_w(const bf16 *a, const float *gup, float *dw, float *db, pgb_lvgeom g)
{
   __shared__ float red[256];
   const int t = blockIdx.y;
   const long o = (t / 9 - 1) * g.plane + ((t / 3) % 3 - 1) * (long)g.Wp + (t % 3 - 1);
   const long nv = (long)g.W * g.H * g.D;
   float acc[16], ab = 0.f;
#pragma unroll
   for (int c = 0; c < 16; c++) acc[c] = 0.f;
   for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < (int)nv; q += gridDim.x * blockDim.x) {
      int x, y, z;
      xyz(q, g, x, y, z);
      const float gv = gup[q];
      const long p = vox(g, x, y, z) + o;
      float v[8];
#pragma unroll
      for (int cb = 0; cb < 2; cb++) {
         load8(a, (long)cb * g.vtot + p, v);
#pragma unroll
         for (int e = 0; e < 8; e++) acc[cb * 8 + e] = fmaf(v[e], gv, acc[cb * 8 + e]);
      }
      ab += gv;
   }
#pragma unroll
   for (int c = 0; c < 16; c++) block_add(acc[c], red, &dw[t * 16 + c]);
   block_add(ab, red, t == 13 ? db : 0);
}

/* first layer dW: dw[t][c] += sum_v s_in rho[v + off t] gz[v][c], db[c] += sum gz */
__global__ void k_in_bwd_w(const float *r32, const bf16 *gz, float *dw, float *db, pgb_lvgeom g)
{
   __shared__ float red[256];
   const int t = blockIdx.y;
   const int ox = t % 3 - 1, oy = (t / 3) % 3 - 1, oz = t / 9 - 1;
   const long nv = (long)g.W * g.H * g.D;
   float acc[16], ab[16];
#pragma unroll
   for (int c = 0; c < 16; c++) acc[c] = ab[c] = 0.f;
   for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < (int)nv; q += gridDim.x * blockDim.x) {
      int x, y, z;
      xyz(q, g, x, y, z);
      const long p = vox(g, x, y, z);
      const float r = r32[p + oz * g.plane + oy * (long)g.Wp + ox];   /* zero on the padding */
      float v[8];
#pragma unroll
      for (int cb = 0; cb < 2; cb++) {
         load8(gz, (long)cb * g.vtot + p, v);
#pragma unroll
         for (int e = 0; e < 8; e++) {
            acc[cb * 8 + e] = fmaf(r, v[e], acc[cb * 8 + e]);
            ab[cb * 8 + e] += v[e];
         }
      }
   }
#pragma unroll
   for (int c = 0; c < 16; c++) block_add(acc[c], red, &dw[t * 16 + c]);
#pragma unroll
   for (int c = 0; c < 16; c++) block_add(ab[c], red, t == 13 ? &db[c] : 0);
}

/* g = g * leaky'(y) (1 where y > 0, else LEAK) over the interior voxels of
 * all channel blocks */
__global__ void k_relu_bwd(bf16 *gv, const bf16 *y, int nch, pgb_lvgeom g)
{
   const long nv = (long)g.W * g.H * g.D, n = nv * (nch / 8);
   for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < (int)n; q += gridDim.x * blockDim.x) {
      const int cb = q / (int)nv, r = q - cb * (int)nv;
      const int x = (int)(r % g.W), yy = (int)((r / g.W) % g.H), z = (int)(r / ((long)g.W * g.H));
      const long idx = cb * g.vtot + vox(g, x, yy, z);
      float a[8], b[8];
      load8(gv, idx, a);
      load8(y, idx, b);
#pragma unroll
      for (int e = 0; e < 8; e++) a[e] = b[e] > 0.f ? a[e] : LEAK * a[e];
      store8(gv, idx, a);
   }
}

/* 2x2x2 average pool (fine f -> coarse c); backward: f += c/8 on the eight
 * children */
__global__ void k_pool(bf16 *f, bf16 *c, int nch, pgb_lvgeom gf, pgb_lvgeom gc, int backward)
{
   const long nv = (long)gc.W * gc.H * gc.D, n = nv * (nch / 8);
   for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < (int)n; q += gridDim.x * blockDim.x) {
      const int cb = q / (int)nv, r = q - cb * (int)nv;
      const int x = (int)(r % gc.W), y = (int)((r / gc.W) % gc.H), z = (int)(r / ((long)gc.W * gc.H));
      const long ic = cb * gc.vtot + vox(gc, x, y, z);
      float s[8], v[8];
      if (!backward) {
#pragma unroll
         for (int e = 0; e < 8; e++) s[e] = 0.f;
         for (int k = 0; k < 8; k++) {
            load8(f, cb * gf.vtot + vox(gf, 2 * x + (k & 1), 2 * y + ((k >> 1) & 1), 2 * z + (k >> 2)), v);
#pragma unroll
            for (int e = 0; e < 8; e++) s[e] += v[e];
         }
#pragma unroll
         for (int e = 0; e < 8; e++) s[e] *= 0.125f;
         store8(c, ic, s);
      } else {
         load8(c, ic, s);
         for (int k = 0; k < 8; k++) {
            const long i = cb * gf.vtot + vox(gf, 2 * x + (k & 1), 2 * y + ((k >> 1) & 1), 2 * z + (k >> 2));
            load8(f, i, v);
#pragma unroll
            for (int e = 0; e < 8; e++) v[e] += 0.125f * s[e];
            store8(f, i, v);
         }
      }
   }
}

/* nearest upsample + skip: out(fine) = up(c) + skip. backward: out (coarse)
 * = sum over the eight children of c (the fine gradient) */
__global__ void k_up(const bf16 *c, const bf16 *skip, bf16 *out, int nch, pgb_lvgeom gf, pgb_lvgeom gc, int backward)
{
   if (!backward) {
      const long nv = (long)gf.W * gf.H * gf.D, n = nv * (nch / 8);
      for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < (int)n; q += gridDim.x * blockDim.x) {
         const int cb = q / (int)nv, r = q - cb * (int)nv;
         const int x = (int)(r % gf.W), y = (int)((r / gf.W) % gf.H), z = (int)(r / ((long)gf.W * gf.H));
         const long i = cb * gf.vtot + vox(gf, x, y, z);
         float a[8], b[8];
         load8(c, cb * gc.vtot + vox(gc, x >> 1, y >> 1, z >> 1), a);
         load8(skip, i, b);
#pragma unroll
         for (int e = 0; e < 8; e++) a[e] += b[e];
         store8(out, i, a);
      }
   } else {
      const long nv = (long)gc.W * gc.H * gc.D, n = nv * (nch / 8);
      for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < (int)n; q += gridDim.x * blockDim.x) {
         const int cb = q / (int)nv, r = q - cb * (int)nv;
         const int x = (int)(r % gc.W), y = (int)((r / gc.W) % gc.H), z = (int)(r / ((long)gc.W * gc.H));
         float s[8] = {0, 0, 0, 0, 0, 0, 0, 0}, v[8];
         for (int k = 0; k < 8; k++) {
            load8(c, cb * gf.vtot + vox(gf, 2 * x + (k & 1), 2 * y + ((k >> 1) & 1), 2 * z + (k >> 2)), v);
#pragma unroll
            for (int e = 0; e < 8; e++) s[e] += v[e];
         }
         store8(out, cb * gc.vtot + vox(gc, x, y, z), s);
      }
   }
}

/* a += b over the interior (skip-connection gradients) */
__global__ void k_add(bf16 *a, const bf16 *b, int nch, pgb_lvgeom g)
{
   const long nv = (long)g.W * g.H * g.D, n = nv * (nch / 8);
   for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < (int)n; q += gridDim.x * blockDim.x) {
      const int cb = q / (int)nv, r = q - cb * (int)nv;
      const int x = (int)(r % g.W), y = (int)((r / g.W) % g.H), z = (int)(r / ((long)g.W * g.H));
      const long i = cb * g.vtot + vox(g, x, y, z);
      float u[8], v[8];
      load8(a, i, u);
      load8(b, i, v);
#pragma unroll
      for (int e = 0; e < 8; e++) u[e] += v[e];
      store8(a, i, u);
   }
}

/* Weight gradient of a tensor-core layer, FP32 on CUDA cores:
 * dw[t][ci][co] += sum_v x[v + off t][ci] * gz[v][co], db[co] += sum gz.
 * blockIdx.y = tap; each thread owns up to 16 (ci, co) pairs; voxels in
 * chunks of WCH staged in shared memory (gz is zero on the padding, so the
 * chunks run over whole padded planes). */
#define WCH 64
__global__ void __launch_bounds__(256) k_conv_bwd_w(const bf16 *x, const bf16 *gz, float *dw, float *db, int cin,
                                                    int cout, pgb_lvgeom g)
{
   extern __shared__ float sh[];
   float *xs = sh, *gs = sh + WCH * cin;
   const int t = blockIdx.y;
   const long o = (t / 9 - 1) * g.plane + ((t / 3) % 3 - 1) * (long)g.Wp + (t % 3 - 1);
   const int npair = cin * cout, per = (npair + 255) / 256;   /* <= 16 */
   float acc[16], ab = 0.f;
#pragma unroll
   for (int k = 0; k < 16; k++) acc[k] = 0.f;
   const long total = (long)g.D * g.plane;
   for (long base = (long)blockIdx.x * WCH; base < total; base += (long)gridDim.x * WCH) {
      __syncthreads();
      for (int q = threadIdx.x; q < WCH * (cin / 8 + cout / 8); q += blockDim.x) {
         const int vv = q % WCH, b8 = q / WCH;
         const long P = g.p0 + base + vv;
         float v[8];
         if (base + vv < total) {
            if (b8 < cin / 8) load8(x, (long)b8 * g.vtot + g.margin + P + o, v);
            else load8(gz, (long)(b8 - cin / 8) * g.vtot + g.margin + P, v);
         } else
            for (int e = 0; e < 8; e++) v[e] = 0.f;
         float *d = b8 < cin / 8 ? xs + vv * cin + b8 * 8 : gs + vv * cout + (b8 - cin / 8) * 8;
         for (int e = 0; e < 8; e++) d[e] = v[e];
      }
      __syncthreads();
#pragma unroll
      for (int k = 0; k < 16; k++) {
         const int pr = threadIdx.x + k * 256;
         if (k >= per || pr >= npair) break;
         const int ci = pr / cout, co = pr % cout;
         float s = acc[k];
         for (int vv = 0; vv < WCH; vv++) s = fmaf(xs[vv * cin + ci], gs[vv * cout + co], s);
         acc[k] = s;
      }
      if (t == 13 && (int)threadIdx.x < cout)
         for (int vv = 0; vv < WCH; vv++) ab += gs[vv * cout + threadIdx.x];
   }
#pragma unroll
   for (int k = 0; k < 16; k++) {
      const int pr = threadIdx.x + k * 256;
      if (k < per && pr < npair) atomicAdd(&dw[((long)t * cin + pr / cout) * cout + pr % cout], acc[k]);
   }
   if (t == 13 && (int)threadIdx.x < cout) atomicAdd(&db[threadIdx.x], ab);
}

/* Adam on FP32 parameters */
__global__ void k_adam(float *w, const float *gw, float *m, float *v, long n, float lr, float b1, float b2,
                       float c1, float c2, float eps)
{
   for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < (int)n; q += gridDim.x * blockDim.x) {
      const float gq = gw[q];
      const float mq = b1 * m[q] + (1.f - b1) * gq, vq = b2 * v[q] + (1.f - b2) * gq * gq;
      m[q] = mq;
      v[q] = vq;
      w[q] -= lr * (mq * c1) / (sqrtf(vq * c2) + eps);
   }
}

/* ------------------------------------------------------ the network (host) -- */
/* NLEV-level encoder-decoder on an (n-1)^3 volume (points 0..n-2 of an n^3
 * grid), levels halving down to (n-1)/32 points a side so that the
 * coarsest convolutions see the whole volume (the solution of the Poisson
 * equation at a point depends on the source everywhere). LCH[v] channels
 * on level v; two 3x3x3 convolutions per encoder level (one after the
 * input convolution on level 0), 2x2x2 average pooling down, nearest
 * upsampling plus the encoder's activation (additive skip) up, one
 * convolution per decoder level, leaky ReLU after every convolution but the
 * last. The first (1 -> 16) and last (16 -> 1) convolutions run on CUDA
 * cores, the others on the tensor cores (forward, and backward-data
 * through the adjoint image).
 *
 * Tensor-core layers in parameter order: 0 = level 0 encoder; 2v-1, 2v =
 * level v encoder (LCH[v-1] -> LCH[v], LCH[v] -> LCH[v]); then the decoder
 * from level NLEV-2 up to 0, level v mapping LCH[v] -> LCH[max(v-1, 0)] so
 * that its output adds onto the skip of level v-1. */
enum { NLEV = 6, NTC = 3 * NLEV - 2 };
static const int LCH[NLEV] = {16, 32, 64, 64, 64, 64};
static int TC_LEV[NTC], TC_CIN[NTC], TC_COUT[NTC];
static int dec_layer(int v) { return 2 * (NLEV - 1) + 1 + (NLEV - 2 - v); }

static void layer_table()
{
   TC_LEV[0] = 0, TC_CIN[0] = TC_COUT[0] = LCH[0];
   for (int v = 1; v < NLEV; v++) {
      TC_LEV[2 * v - 1] = TC_LEV[2 * v] = v;
      TC_CIN[2 * v - 1] = LCH[v - 1];
      TC_COUT[2 * v - 1] = TC_CIN[2 * v] = TC_COUT[2 * v] = LCH[v];
   }
   for (int v = NLEV - 2; v >= 0; v--) {
      const int l = dec_layer(v);
      TC_LEV[l] = v;
      TC_CIN[l] = LCH[v];
      TC_COUT[l] = LCH[v > 0 ? v - 1 : 0];
   }
}

/* activations per level: E0, E1 (encoder), P (pooled input, v >= 1), C
 * (upsampled decoder + skip, v <= NLEV-2), D (decoder output, v <= NLEV-2) */
enum { K_E0, K_E1, K_P, K_C, K_D, NKIND };
enum { NACT = NKIND * NLEV };
static int act_id(int kind, int v) { return kind * NLEV + v; }

static int act_ch(int kind, int v)
{
   if (kind == K_P) return LCH[v - 1];
   if (kind == K_D) return LCH[v > 0 ? v - 1 : 0];
   return LCH[v];
}

static bool act_used(int kind, int v)
{
   return !((kind == K_P && v == 0) || ((kind == K_C || kind == K_D) && v == NLEV - 1));
}

struct pgb_net {
   int n;
   pgb_lvgeom g[NLEV];
   double s_in, s_out;
   const double *d_q;             /* while set: the charge the scales come from, on the device */
   double q_gain;                 /* s_out = q_gain * charge then */
   long np;                       /* parameter count */
   float *p, *gp, *m, *v;         /* parameters, gradients, Adam moments */
   long off_tc_w[NTC], off_tc_b[NTC], off_in_w, off_in_b, off_out_w, off_out_b;
   bf16 *img[NTC], *img_adj[NTC];
   bf16 *act[NACT], *grad[NACT];
   float *up, *gup, *r32;
   double *d_loss;
   double *d_dots;                /* energy-norm scaling sums, and the count of rejected guesses */
   int *d_err;
   long step;
   int bias_free;
};

static size_t act_bytes(const pgb_lvgeom &g, int ch) { return (size_t)(ch / 8) * g.vtot * 16; }

static uint64_t splitmix(uint64_t *s)
{
   uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
   z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
   z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
   return z ^ (z >> 31);
}

static double gauss(uint64_t *s)
{
   double u1 = ((splitmix(s) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
   double u2 = ((splitmix(s) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
   return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

static int repack(pgb_net *net, cudaStream_t st)
{
   for (int l = 0; l < NTC; l++) {
      const float *w = net->p + net->off_tc_w[l];
      if (pgb_conv3d_pack_weights(w, net->img[l], TC_CIN[l], TC_COUT[l], 0, st) ||
          pgb_conv3d_pack_weights(w, net->img_adj[l], TC_CIN[l], TC_COUT[l], 1, st))
         return 11;
   }
   return 0;
}

extern "C" void pgb_net_destroy(pgb_net *net)
{
   if (!net) return;
   cudaFree(net->p);
   cudaFree(net->gp);
   cudaFree(net->m);
   cudaFree(net->v);
   for (int l = 0; l < NTC; l++) {
      cudaFree(net->img[l]);
      cudaFree(net->img_adj[l]);
   }
   for (int a = 0; a < NACT; a++) {
      cudaFree(net->act[a]);
      cudaFree(net->grad[a]);
   }
   cudaFree(net->up);
   cudaFree(net->gup);
   cudaFree(net->r32);
   cudaFree(net->d_loss);
   cudaFree(net->d_dots);
   cudaFree(net->d_err);
   free(net);
}

extern "C" int pgb_net_create(int n, unsigned long long seed, pgb_net **out)
{
   *out = 0;
   const int step = 1 << (NLEV - 1);
   if (n < 2 * step + 1 || (n - 1) % step != 0 || n > 513)
      return arg_err("pgb_net_create: n-1 must be a multiple of 32, 65 <= n <= 513");
   layer_table();
   pgb_net *net = (pgb_net *)calloc(1, sizeof(pgb_net));
   if (!net) return arg_err("pgb_net_create: out of host memory");
   net->n = n;
   net->s_in = net->s_out = 1.0;
   for (int l = 0; l < NLEV; l++) {
      const int e = (n - 1) >> l;
      net->g[l] = make_geom(e, e, e);
   }
   long o = 0;
   net->off_in_w = o; o += 27 * LCH[0];
   net->off_in_b = o; o += LCH[0];
   for (int l = 0; l < NTC; l++) {
      net->off_tc_w[l] = o; o += 27L * TC_CIN[l] * TC_COUT[l];
      net->off_tc_b[l] = o; o += TC_COUT[l];
   }
   net->off_out_w = o; o += 27 * LCH[0];
   net->off_out_b = o; o += 1;
   net->np = o;
   const size_t nv = (size_t)(n - 1) * (n - 1) * (n - 1);
   bool ok = cudaMalloc((void **)&net->p, o * 4) == cudaSuccess && cudaMalloc((void **)&net->gp, o * 4) == cudaSuccess &&
             cudaMalloc((void **)&net->m, o * 4) == cudaSuccess && cudaMalloc((void **)&net->v, o * 4) == cudaSuccess &&
             cudaMalloc((void **)&net->up, nv * 4) == cudaSuccess && cudaMalloc((void **)&net->gup, nv * 4) == cudaSuccess &&
             cudaMalloc((void **)&net->r32, net->g[0].vtot * 4) == cudaSuccess &&
             cudaMemset(net->r32, 0, net->g[0].vtot * 4) == cudaSuccess &&
             cudaMalloc((void **)&net->d_loss, 8) == cudaSuccess && cudaMalloc((void **)&net->d_err, 4) == cudaSuccess &&
             cudaMalloc((void **)&net->d_dots, 24) == cudaSuccess && cudaMemset(net->d_dots, 0, 24) == cudaSuccess;
   for (int l = 0; l < NTC && ok; l++)
      ok = cudaMalloc((void **)&net->img[l], 27L * TC_CIN[l] * TC_COUT[l] * 2) == cudaSuccess &&
           cudaMalloc((void **)&net->img_adj[l], 27L * TC_CIN[l] * TC_COUT[l] * 2) == cudaSuccess;
   for (int k = 0; k < NKIND && ok; k++)
      for (int v = 0; v < NLEV && ok; v++) {
         if (!act_used(k, v)) continue;
         const int a = act_id(k, v);
         const size_t b = act_bytes(net->g[v], act_ch(k, v));
         ok = cudaMalloc((void **)&net->act[a], b) == cudaSuccess && cudaMalloc((void **)&net->grad[a], b) == cudaSuccess &&
              cudaMemset(net->act[a], 0, b) == cudaSuccess && cudaMemset(net->grad[a], 0, b) == cudaSuccess;
      }
   if (!ok) {
      pgb_net_destroy(net);
      return arg_err("pgb_net_create: device allocation failed");
   }
   /* He-normal weights (the last layer scaled down), zero biases */
   float *h = (float *)calloc(o, 4);
   uint64_t s = seed ? seed : 1;
   for (int k = 0; k < 27 * LCH[0]; k++) h[net->off_in_w + k] = (float)(gauss(&s) * sqrt(2.0 / 27.0));
   for (int l = 0; l < NTC; l++)
      for (long k = 0; k < 27L * TC_CIN[l] * TC_COUT[l]; k++)
         h[net->off_tc_w[l] + k] = (float)(gauss(&s) * sqrt(2.0 / (27.0 * TC_CIN[l])));
   for (int k = 0; k < 27 * LCH[0]; k++)
      h[net->off_out_w + k] = (float)(0.1 * gauss(&s) * sqrt(1.0 / (27.0 * LCH[0])));
   cudaMemcpy(net->p, h, o * 4, cudaMemcpyHostToDevice);
   free(h);
   cudaMemset(net->m, 0, o * 4);
   cudaMemset(net->v, 0, o * 4);
   cudaMemset(net->d_err, 0, 4);
   if (repack(net, 0)) {
      pgb_net_destroy(net);
      return 11;
   }
   *out = net;
   return 0;
}

extern "C" int pgb_net_set_scales(pgb_net *net, double s_in, double s_out)
{
   net->s_in = s_in;
   net->s_out = s_out;
   return 0;
}

/* the bias entries of the parameter vector: (offset, count) pairs */
static int bias_ranges(const pgb_net *net, long *off, long *cnt)
{
   int k = 0;
   off[k] = net->off_in_b, cnt[k++] = LCH[0];
   for (int l = 0; l < NTC; l++) off[k] = net->off_tc_b[l], cnt[k++] = TC_COUT[l];
   off[k] = net->off_out_b, cnt[k++] = 1;
   return k;
}

/* on = 1 holds every bias at zero (set now, gradients dropped before each
 * Adam step): the net is then positively homogeneous, net(c rho) = c
 * net(rho) for c > 0, which is what a guess of a linear equation's
 * solution should be */
/* at most `ctas` CTAs for the persistent (z-marching) convolution of every
 * net in the process, 0 for a full wave; results do not depend on it */
extern "C" int pgb_net_set_grid_cap(int ctas)
{
   if (ctas < 0) return arg_err("pgb_net_set_grid_cap: negative");
   g_tcz_cap = ctas;
   return 0;
}

extern "C" int pgb_net_set_bias_free(pgb_net *net, int on)
{
   net->bias_free = on;
   if (!on) return 0;
   long off[NTC + 2], cnt[NTC + 2];
   const int k = bias_ranges(net, off, cnt);
   for (int i = 0; i < k; i++)
      if (cudaMemset(net->p + off[i], 0, cnt[i] * 4) != cudaSuccess ||
          cudaMemset(net->m + off[i], 0, cnt[i] * 4) != cudaSuccess ||
          cudaMemset(net->v + off[i], 0, cnt[i] * 4) != cudaSuccess)
         return arg_err("pgb_net_set_bias_free: clearing the biases failed");
   return 0;
}

extern "C" long pgb_net_num_params(pgb_net *net) { return net->np; }

/* which = 0 parameters, 1 gradients; to_device = 1 uploads (parameters) */
extern "C" int pgb_net_params(pgb_net *net, int which, float *host, int to_device)
{
   float *d = which ? net->gp : net->p;
   cudaError_t e = to_device ? cudaMemcpy(d, host, net->np * 4, cudaMemcpyHostToDevice)
                             : cudaMemcpy(host, d, net->np * 4, cudaMemcpyDeviceToHost);
   if (e != cudaSuccess) return arg_err("pgb_net_params: copy failed");
   if (to_device && !which) return repack(net, 0);
   return 0;
}

#define GRID_1D 1216
#define NETK(call, name)                 \
   do {                                  \
      call;                              \
      if (check_net(name)) return 11;    \
   } while (0)

static int tc(pgb_net *net, int l, const bf16 *in, bf16 *out, int adjoint, cudaStream_t st)
{
   const pgb_lvgeom &g = net->g[TC_LEV[l]];
   if (!adjoint)
      return conv_dispatch(TC_CIN[l], TC_COUT[l], in, out, net->img[l], net->p + net->off_tc_b[l], g, 1,
                           net->d_err, st);
   return conv_dispatch(TC_COUT[l], TC_CIN[l], in, out, net->img_adj[l], 0, g, 0, net->d_err, st);
}

/* what level v's upsampling reads: the coarsest encoder output for the
 * level above the bottom, else the decoder output of level v+1 */
static int coarse_src(int v) { return v + 1 == NLEV - 1 ? act_id(K_E1, NLEV - 1) : act_id(K_D, v + 1); }

static int forward(pgb_net *net, const double *rho, cudaStream_t st)
{
   bf16 **a = net->act;
   pgb_lvgeom *g = net->g;
#define A(k, v) a[act_id(k, v)]
   NETK((k_rho32<<<GRID_1D, 256, 0, st>>>(rho, net->n, (float)net->s_in, net->d_q, net->r32, g[0])), "net rho32");
   NETK((k_in_fwd<<<(g[0].W * g[0].H * g[0].D + 255) / 256, 256, 0, st>>>(net->r32, net->p + net->off_in_w,
                                                                          net->p + net->off_in_b, A(K_E0, 0), g[0])),
        "net in");
   if (tc(net, 0, A(K_E0, 0), A(K_E1, 0), 0, st)) return 11;
   for (int v = 1; v < NLEV; v++) {
      NETK((k_pool<<<GRID_1D, 256, 0, st>>>(A(K_E1, v - 1), A(K_P, v), LCH[v - 1], g[v - 1], g[v], 0)), "net pool");
      if (tc(net, 2 * v - 1, A(K_P, v), A(K_E0, v), 0, st) || tc(net, 2 * v, A(K_E0, v), A(K_E1, v), 0, st))
         return 11;
   }
   for (int v = NLEV - 2; v >= 0; v--) {
      NETK((k_up<<<GRID_1D, 256, 0, st>>>(a[coarse_src(v)], A(K_E1, v), A(K_C, v), LCH[v], g[v], g[v + 1], 0)),
           "net up");
      if (tc(net, dec_layer(v), A(K_C, v), A(K_D, v), 0, st)) return 11;
   }
   NETK((k_out_fwd<<<GRID_1D, 256, 0, st>>>(A(K_D, 0), net->p + net->off_out_w, net->p + net->off_out_b, net->up,
                                             g[0])), "net out");
#undef A
   return 0;
}

extern "C" int pgb_net_predict(pgb_net *net, const double *rho, double *u, void *stream)
{
   cudaStream_t st = (cudaStream_t)stream;
   if (forward(net, rho, st)) return 11;
   NETK((k_out_store<<<GRID_1D, 256, 0, st>>>(net->up, u, net->n, net->s_out, net->d_q, net->q_gain, net->g[0])),
        "net store");
   return 0;
}

/* pgb_net_predict with the input and output scales taken from the source's
 * charge q (a device value, e.g. h^3 sum |rho|, computed on the same stream):
 * s_in = 1/q, s_out = gain q, so that the host never waits for the charge */
extern "C" int pgb_net_predict_charge(pgb_net *net, const double *rho, double *u, const double *q, double gain,
                                      void *stream)
{
   if (!q) return arg_err("pgb_net_predict_charge: no charge");
   net->d_q = q;
   net->q_gain = gain;
   const int rc = pgb_net_predict(net, rho, u, stream);
   net->d_q = 0;
   return rc;
}

extern "C" int pgb_net_rescale(pgb_net *net, const double *rho, double *u, double h, void *stream)
{
   cudaStream_t st = (cudaStream_t)stream;
   if (!(h > 0)) return arg_err("pgb_net_rescale: spacing must be positive");
   if (cudaMemsetAsync(net->d_dots, 0, 16, st) != cudaSuccess) return check_net("net memset");   /* keeps dots[2] */
   const long nn = (long)net->n * net->n * net->n;
   NETK((k_energy_dots<<<GRID_1D, 256, 0, st>>>(rho, u, net->n, 1.0 / (h * h), net->d_dots)), "net energy dots");
   NETK((k_scale_guess<<<GRID_1D, 256, 0, st>>>(u, nn, net->d_dots)), "net scale guess");
   return 0;
}

static int wgrad(pgb_net *net, int l, const bf16 *x, const bf16 *gz, cudaStream_t st)
{
   const pgb_lvgeom &g = net->g[TC_LEV[l]];
   const long chunks = ((long)g.D * g.plane + WCH - 1) / WCH;
   const int nblk = (int)(chunks < 96 ? chunks : 96);
   const size_t sh = (size_t)WCH * (TC_CIN[l] + TC_COUT[l]) * 4;
   NETK((k_conv_bwd_w<<<dim3(nblk, 27), 256, sh, st>>>(x, gz, net->gp + net->off_tc_w[l], net->gp + net->off_tc_b[l],
                                                         TC_CIN[l], TC_COUT[l], g)),
        "net wgrad");
   return 0;
}

/* backward of one activated convolution x -> y: the gradient of y (taken
 * through the activation in place) gives the weight gradient and the
 * gradient of x */
static int conv_bwd(pgb_net *net, int l, int x, int y, cudaStream_t st)
{
   bf16 **a = net->act, **G = net->grad;
   NETK((k_relu_bwd<<<GRID_1D, 256, 0, st>>>(G[y], a[y], TC_COUT[l], net->g[TC_LEV[l]])), "net relu");
   if (wgrad(net, l, a[x], G[y], st) || tc(net, l, G[y], G[x], 1, st)) return 11;
   return 0;
}

/* loss and gradients of all parameters for one (rho, u) pair */
static int loss_grad(pgb_net *net, const double *rho, const float *ut, cudaStream_t st)
{
   bf16 **a = net->act, **G = net->grad;
   pgb_lvgeom *g = net->g;
   if (forward(net, rho, st)) return 11;
   if (cudaMemsetAsync(net->gp, 0, net->np * 4, st) != cudaSuccess ||
       cudaMemsetAsync(net->d_loss, 0, 8, st) != cudaSuccess)
      return check_net("net memset");
   /* the encoder outputs above the bottom take gradients along two paths
    * (skip and pooling): they accumulate from zero */
   for (int v = 0; v < NLEV - 1; v++)
      if (cudaMemsetAsync(G[act_id(K_E1, v)], 0, act_bytes(g[v], LCH[v]), st) != cudaSuccess)
         return check_net("net memset");
   NETK((k_loss<<<GRID_1D, 256, 0, st>>>(net->up, ut, net->n, (float)(1.0 / net->s_out), net->gup, net->d_loss, g[0])),
        "net loss");
   const int d0 = act_id(K_D, 0);
   NETK((k_out_bwd_w<<<dim3(96, 27), 256, 0, st>>>(a[d0], net->gup, net->gp + net->off_out_w, net->gp + net->off_out_b,
                                                    g[0])), "net out w");
   NETK((k_out_bwd_data<<<GRID_1D, 256, 0, st>>>(net->gup, net->p + net->off_out_w, G[d0], g[0])), "net out data");
   /* decoder, fine to coarse */
   for (int v = 0; v <= NLEV - 2; v++) {
      const int c = act_id(K_C, v);
      if (conv_bwd(net, dec_layer(v), c, act_id(K_D, v), st)) return 11;
      NETK((k_add<<<GRID_1D, 256, 0, st>>>(G[act_id(K_E1, v)], G[c], LCH[v], g[v])), "net add");
      NETK((k_up<<<GRID_1D, 256, 0, st>>>(G[c], 0, G[coarse_src(v)], LCH[v], g[v], g[v + 1], 1)), "net up bwd");
   }
   /* encoder, coarse to fine */
   for (int v = NLEV - 1; v >= 1; v--) {
      const int p = act_id(K_P, v);
      if (conv_bwd(net, 2 * v, act_id(K_E0, v), act_id(K_E1, v), st) ||
          conv_bwd(net, 2 * v - 1, p, act_id(K_E0, v), st))
         return 11;
      NETK((k_pool<<<GRID_1D, 256, 0, st>>>(G[act_id(K_E1, v - 1)], G[p], LCH[v - 1], g[v - 1], g[v], 1)),
           "net pool bwd");
   }
   const int e0 = act_id(K_E0, 0);
   if (conv_bwd(net, 0, e0, act_id(K_E1, 0), st)) return 11;
   NETK((k_relu_bwd<<<GRID_1D, 256, 0, st>>>(G[e0], a[e0], LCH[0], g[0])), "net relu");
   NETK((k_in_bwd_w<<<dim3(96, 27), 256, 0, st>>>(net->r32, G[e0], net->gp + net->off_in_w,
                                                   net->gp + net->off_in_b, g[0])), "net in w");
   return 0;
}

static int read_loss(pgb_net *net, double *loss, cudaStream_t st)
{
   int e = 0;
   if (cudaMemcpyAsync(loss, net->d_loss, 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
       cudaMemcpyAsync(&e, net->d_err, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
       cudaStreamSynchronize(st) != cudaSuccess)
      return arg_err("net: reading the loss back failed");
   if (e) return arg_err("net: a wait inside a tensor-core convolution ran out");
   return 0;
}

extern "C" int pgb_net_loss_grad(pgb_net *net, const double *rho, const float *ut, double *loss, void *stream)
{
   cudaStream_t st = (cudaStream_t)stream;
   if (loss_grad(net, rho, ut, st)) return 11;
   return read_loss(net, loss, st);
}

extern "C" int pgb_net_train_step(pgb_net *net, const double *rho, const float *ut, float lr, double *loss,
                                  void *stream)
{
   cudaStream_t st = (cudaStream_t)stream;
   if (loss_grad(net, rho, ut, st)) return 11;
   if (net->bias_free) {
      long off[NTC + 2], cnt[NTC + 2];
      const int k = bias_ranges(net, off, cnt);
      for (int i = 0; i < k; i++)
         if (cudaMemsetAsync(net->gp + off[i], 0, cnt[i] * 4, st) != cudaSuccess) return check_net("net memset");
   }
   net->step++;
   const float b1 = 0.9f, b2 = 0.999f;
   const float c1 = (float)(1.0 / (1.0 - pow(b1, (double)net->step)));
   const float c2 = (float)(1.0 / (1.0 - pow(b2, (double)net->step)));
   NETK((k_adam<<<GRID_1D, 256, 0, st>>>(net->p, net->gp, net->m, net->v, net->np, lr, b1, b2, c1, c2, 1e-8f)),
        "net adam");
   if (repack(net, st)) return 11;
   return loss ? read_loss(net, loss, st) : 0;
}

/* how many guesses pgb_net_rescale has replaced by u = 0 so far */
extern "C" int pgb_net_rejected_guesses(pgb_net *net, long *count)
{
   double v = 0;
   if (cudaMemcpy(&v, net->d_dots + 2, sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
      return check_net("net rejected count");
   *count = (long)v;
   return 0;
}

