/*
 * pearson_gemm.cu -- pairwise-complete Pearson for clusmethod none as a dense
 * masked contraction on the tcgen05 tensor cores (precision 1 TF32, 2 3xBF16,
 * 4 scaled FP16), and the same contraction tiled on the CUDA cores in FP32
 * (precision 3, the comparator for the tensor-core forms).
 *
 * For genes x, y with usable-sample masks m and centred values a (a = v - mean
 * over the gene's usable samples, 0 where unusable), every sum Pearson needs
 * over the samples both genes have is a product of two [genes][samples]
 * operands:
 *     n   = M  . M^T      Sxy = A . A^T
 *     Sx  = A  . M^T      Sy  = M . A^T
 *     Sxx = A2 . M^T      Syy = M . A2^T       (A2 = a^2)
 * Centring by the gene mean changes no correlation (r is shift invariant per
 * gene) but removes the cancellation that would otherwise swamp TF32.  A CTA
 * computes 128 x 64 tiles of pairs: TMA streams swizzled K-chunks of the
 * operands into a 3-stage shared-memory ring, one thread issues the
 * tcgen05.mma instructions (M = 128) into six 64-column accumulators held in
 * TMEM (384 of the 512 columns), and eight warps read them back with
 * tcgen05.ld and form r = (n Sxy - Sx Sy) / sqrt((n Sxx - Sx^2)(n Syy - Sy^2))
 * with error-compensated products.  3xBF16 splits a = hi + lo and sums
 * hi.hi + hi.lo + lo.hi (the mask is exact in BF16).  FP16 (precision 4) scales each gene's
 * centred values by a power of two so that the largest |a| is at most 1, which leaves r unchanged
 * (r is scale invariant per gene, and a power of two scales exactly), and rounds a, a^2 and m to
 * FP16: the same 11-bit significand as TF32, two bytes instead of four, and twice the MMA rate, so
 * a 128-byte row of a K-chunk holds 64 samples instead of 32.  Values below 2^-14 of a gene's
 * largest |a| (squares below 2^-14 of its largest square) keep fewer significant bits.
 *
 * The result is the mathematically pairwise-complete Pearson (each sample's own
 * values), i.e. semantics "fixed"; KINC's packed-array indexing is not a
 * contraction.  Every wait on an mbarrier is bounded: on expiry the kernel
 * records an error, drains its own copies (bounded), frees its TMEM and returns.
 */
#include "../../include/kinc_sim.h"
#include "pearson_tc.h"

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>

namespace kinc_tc {

constexpr int BM = 128;               /* pair-tile rows (genes x) */
constexpr int NACC = 6;               /* Sxy, Sx, Sy, Sxx, Syy, n */
constexpr int TMEM_COLS = 512;
constexpr long long WAIT_CYCLES = 4ll << 30;  /* ~2 s of SM clock before a wait gives up */

constexpr int ST_TIMEOUT = 10;        /* an mbarrier wait expired */

/* warps of a tensor-core CTA: producer, MMA issuer, then two epilogue warps per TMEM lane quarter */
constexpr int EPI_WARPS = 8;
constexpr int TC_THREADS = (2 + EPI_WARPS) * 32;

/* per precision: element type, elements per K-chunk row, swizzle, operands per side */
template <int MODE> struct Cfg;
/*
 * Tiles are 128 x 64 pairs.  (128 x 80 TF32 tiles -- 480 TMEM columns, 16-sample chunks in a
 * 5-stage ring of 64-byte rows -- were measured slower: 8.44 against 6.97 ms for the 20,000 x 2,000
 * matrix.)
 */
#ifndef KINC_TC_PAIR
#define KINC_TC_PAIR 0                /* 1: TF32 on CTA pairs (cta_group::2, M = 256): bit-identical
                                         results, measured 3.5 % slower on 134M-pair blocks (4.63 vs
                                         4.47 ms) and 20 % slower on 4M-pair blocks */
#endif
#ifndef KINC_TC_TF32_BK16
#define KINC_TC_TF32_BK16 0           /* 1: TF32 K-chunks of 16 samples (64-byte rows) in a 6-stage ring:
                                         measured slower, 8.2-8.6 vs 6.6-7.0 ms per 134M-pair block */
#endif
template <> struct Cfg<1>             /* TF32: A, A2, M as fp32 rounded to tf32 */
{
   static constexpr int ELEM = 4;
   static constexpr int BN = 64;      /* pair-tile columns (genes y) */
#if KINC_TC_TF32_BK16
   static constexpr int BK = 16;      /* 64-byte rows, SWIZZLE_64B */
   static constexpr int ROWB = 64;
   static constexpr int STAGES = 6;
   static constexpr uint64_t LAYOUT = 4;              /* SWIZZLE_64B */
#else
   static constexpr int BK = 32;      /* 128-byte rows, SWIZZLE_128B */
   static constexpr int ROWB = 128;
   static constexpr int STAGES = 3;
   static constexpr uint64_t LAYOUT = 2;              /* SWIZZLE_128B */
#endif
   static constexpr int NMAT = 3;
   static constexpr int UMMA_K = 8;
   static constexpr uint32_t A_FMT = 2, B_FMT = 2;   /* tf32 */
};
template <> struct Cfg<4>             /* FP16: A, A2, M with each gene scaled by a power of two */
{
   static constexpr int ELEM = 2;
   static constexpr int BN = 64;
   static constexpr int BK = 64;      /* 128-byte rows, SWIZZLE_128B */
   static constexpr int ROWB = 128;
   static constexpr int NMAT = 3;
   static constexpr int UMMA_K = 16;
   static constexpr int STAGES = 3;
   static constexpr uint32_t A_FMT = 0, B_FMT = 0;   /* f16 */
   static constexpr uint64_t LAYOUT = 2;              /* SWIZZLE_128B */
};
template <> struct Cfg<2>             /* 3xBF16: A_hi, A_lo, A2_hi, A2_lo, M as bf16 */
{
   static constexpr int ELEM = 2;
   static constexpr int BN = 64;
   static constexpr int BK = 32;      /* 64-byte rows, SWIZZLE_64B */
   static constexpr int ROWB = 64;
   static constexpr int NMAT = 5;
   static constexpr int UMMA_K = 16;
   static constexpr int STAGES = 3;
   static constexpr uint32_t A_FMT = 1, B_FMT = 1;   /* bf16 */
   static constexpr uint64_t LAYOUT = 4;              /* SWIZZLE_64B */
};

template <int MODE>
struct Layout
{
   static constexpr int XMAT = BM * Cfg<MODE>::ROWB;          /* bytes of one x-side operand chunk */
   static constexpr int YMAT = Cfg<MODE>::BN * Cfg<MODE>::ROWB;
   static constexpr int STAGE = Cfg<MODE>::NMAT * (XMAT + YMAT);
   static constexpr int RING = Cfg<MODE>::STAGES * STAGE;
   /* the epilogue warps' transposition tiles: 32 rows x 8 columns of r each */
   static constexpr int EBUF = EPI_WARPS * 32 * 8 * 4;
   static constexpr int SMEM = RING + 1024 /* alignment slack */ + 256 /* barriers */ + EBUF;
   static_assert(SMEM <= 227 * 1024, "ring, barriers and epilogue tiles fit the shared memory of one CTA");
};

/* ---------------------------------------------------------------- PTX */

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
   return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
   asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
   asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

/* bounded wait for phase `parity` of an mbarrier; false on expiry */
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity)
{
   const long long t0 = clock64();
   for ( ;; )
   {
      uint32_t ok;
      asm volatile("{\n\t.reg .pred p;\n\t"
                   "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                   "selp.u32 %0, 1, 0, p;\n\t}"
                   : "=r"(ok)
                   : "r"(bar), "r"(parity)
                   : "memory");
      if ( ok ) return true;
      if ( clock64() - t0 > WAIT_CYCLES ) return false;
   }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar)
{
   asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
                "l"((uint64_t)map), "r"(x), "r"(y), "r"(bar)
                : "memory");
}

__device__ __forceinline__ uint32_t cluster_rank()
{
   uint32_t r;
   asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
   return r;
}

/* every thread of every CTA of the cluster; release/acquire orders shared-memory state across it */
__device__ __forceinline__ void cluster_sync()
{
   asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}

/* shared-memory matrix descriptor: K-major, swizzled rows of ROWB bytes, 8-row atoms */
template <int MODE>
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr)
{
   const uint64_t sbo = (uint64_t)(8 * Cfg<MODE>::ROWB) >> 4;
   uint64_t d = 0;
   d |= (uint64_t)((addr >> 4) & 0x3fff);       /* start address */
   d |= (uint64_t)0 << 16;                        /* leading byte offset: unused for swizzled K-major */
   d |= (sbo & 0x3fff) << 32;                     /* stride byte offset: next 8-row group */
   d |= (uint64_t)1 << 46;                        /* descriptor version */
   d |= Cfg<MODE>::LAYOUT << 61;                  /* swizzle mode */
   return d;
}

/* instruction descriptor: D f32, A/B format, both K-major, N columns, M rows (128 on one CTA,
 * 256 on a CTA pair) */
template <int MODE, int N = Cfg<MODE>::BN, int M = BM>
__host__ __device__ constexpr uint32_t instr_desc()
{
   static_assert(N % 16 == 0 && N >= 16 && N <= 256, "M = 128 and 256 take N in 16..256, a multiple of 16");
   static_assert(M == 128 || M == 256, "M is 128 (one CTA) or 256 (a CTA pair)");
   return (1u << 4)                                /* D format f32 */
          | (Cfg<MODE>::A_FMT << 7) | (Cfg<MODE>::B_FMT << 10)
          | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

/*
 * TF32 and FP16: the six contractions share three x-side operands, so they are issued as three MMAs
 * with the y-side operands stacked along N -- A_x.[A_y; M_y], A2_x.M_y, M_x.[A2_y; A_y; M_y]
 * (N = 128, 64, 192) -- which reads each x-side operand from shared memory once per K step
 * instead of two or three times (with N = 64 the operand reads, not the tensor pipe, bound the
 * MMAs).  The y-side planes sit in shared memory as [A2_y][A_y][M_y] so both stacks are
 * contiguous; the accumulators land in TMEM columns Sxy 0, Sx 64, Sxx 128, Syy 192, Sy 256, n 320.
 */
#ifndef KINC_TC_MERGE
#define KINC_TC_MERGE 1
#endif
/*
 * 3xBF16: twelve products (Sxy = Ah.Ah + Ah.Al + Al.Ah, Sx = Ah.M + Al.M, Sy = M.Ah + M.Al,
 * Sxx = Qh.M + Ql.M, Syy = M.Qh + M.Ql, n = M.M; Q = A2) as seven MMAs: Ah_x.[Ah; M; Al]_y
 * (N = 192), Al_x.[Ah; M]_y accumulated onto its first 128 columns, Qh_x.M_y and Ql_x.M_y,
 * M_x.[Qh; Ah; M]_y (N = 192), M_x.Ql_y and M_x.Al_y accumulated onto the Syy and Sy columns.
 * The y-side planes sit as [Ql][Qh][Ah][M][Al] so every stack is contiguous.  Sxy is kept in two
 * FP32 accumulators (Ah.Ah + Al.Ah in columns 0-63, Ah.Al in 128-191) added in the epilogue;
 * Sx 64, Sxx 192, Syy 256, Sy 320, n 384 (448 of 512 columns).
 */
#ifndef KINC_TC_MERGE_BF16
#define KINC_TC_MERGE_BF16 1
#endif
template <int MODE>
__host__ __device__ constexpr bool merged()
{
   return ((MODE == 1 || MODE == 4) && KINC_TC_MERGE) || (MODE == 2 && KINC_TC_MERGE_BF16);
}

/* shared-memory slot of y-side operand m (TF32: 0 A, 1 A2, 2 M; 3xBF16: 0 Ah, 1 Al, 2 Qh, 3 Ql, 4 M) */
template <int MODE>
__host__ __device__ constexpr int yslot(int m)
{
   return !merged<MODE>() ? m
          : MODE != 2     ? (m == 0 ? 1 : m == 1 ? 0 : 2)
                          : (m == 0 ? 2 : m == 1 ? 4 : m == 2 ? 1 : m == 3 ? 0 : 3);
}

/* TMEM column of accumulator a (0 Sxy, 1 Sx, 2 Sy, 3 Sxx, 4 Syy, 5 n) */
template <int MODE>
__host__ __device__ constexpr int acc_col(int a)
{
   return !merged<MODE>() ? a * Cfg<MODE>::BN
          : MODE != 2     ? (a == 0 ? 0 : a == 1 ? 64 : a == 2 ? 256 : a == 3 ? 128 : a == 4 ? 192 : 320)
                          : (a == 0 ? 0 : a == 1 ? 64 : a == 2 ? 320 : a == 3 ? 192 : a == 4 ? 256 : 384);
}

/* the second Sxy accumulator of merged 3xBF16 (Ah.Al), -1 when there is none */
template <int MODE>
__host__ __device__ constexpr int sxy2_col()
{
   return (merged<MODE>() && MODE == 2) ? 128 : -1;
}

template <int MODE, int N = Cfg<MODE>::BN>
__device__ __forceinline__ void mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate)
{
   constexpr uint32_t idesc = instr_desc<MODE, N>();
   if ( MODE == 1 )
   {
      asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                   "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
                   "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
   }
   else
   {
      asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                   "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
                   "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
   }
}

__device__ __forceinline__ void mma_commit(uint32_t bar)
{
   asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                : "memory");
}

/* ---- CTA-pair (cta_group::2) forms */

/* M = 256 TF32 MMA of a CTA pair, issued by the even CTA: A rows 0-127 and the first N/2 rows of
 * B from its shared memory, rows 128-255 and the other N/2 rows of B from the odd CTA's (same
 * offsets); D rows 0-127 into the even CTA's TMEM, 128-255 into the odd CTA's */
template <int N>
__device__ __forceinline__ void mma_pair_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate)
{
   constexpr uint32_t idesc = instr_desc<1, N, 256>();
   asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                "tcgen05.mma.cta_group::2.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
                "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

/* an arrival on the mbarrier at offset `bar` of every CTA of the pair in `mask` once the pair
 * MMAs issued so far have completed */
__device__ __forceinline__ void commit_pair(uint32_t bar, uint16_t mask)
{
   asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;"
                ::"r"(bar), "h"(mask)
                : "memory");
}

/* a TMA load into this CTA's shared memory that signals the mbarrier `bar_cl` (a cluster address,
 * possibly in the other CTA of the pair) */
__device__ __forceinline__ void tma_load_2d_pair(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar_cl)
{
   asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes.cta_group::2"
                " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
                "l"((uint64_t)map), "r"(x), "r"(y), "r"(bar_cl)
                : "memory");
}

/* the cluster address of this CTA's shared-memory location `addr` in CTA `rank` */
__device__ __forceinline__ uint32_t mapa_rank(uint32_t addr, uint32_t rank)
{
   uint32_t r;
   asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
   return r;
}

__device__ __forceinline__ void mbar_arrive_cluster(uint32_t bar_cl)
{
   asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(bar_cl) : "memory");
}

/* mbar_wait for a barrier that threads of the other CTA arrive on */
__device__ __forceinline__ bool mbar_wait_cluster(uint32_t bar, uint32_t parity)
{
   const long long t0 = clock64();
   for ( ;; )
   {
      uint32_t ok;
      asm volatile("{\n\t.reg .pred p;\n\t"
                   "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
                   "selp.u32 %0, 1, 0, p;\n\t}"
                   : "=r"(ok)
                   : "r"(bar), "r"(parity)
                   : "memory");
      if ( ok ) return true;
      if ( clock64() - t0 > WAIT_CYCLES ) return false;
   }
}

/* 16 consecutive TMEM columns of this warp's 32 lanes into r (asynchronous: tmem_wait_ld before use) */
__device__ __forceinline__ void tmem_ld16_async(uint32_t taddr, uint32_t* r)
{
   asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15},"
                " [%16];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                  "=r"(r[15])
                : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait_ld()
{
   asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

/* ------------------------------------------------------------ kernels */

/* Operands per gene (one warp per gene): mean over usable samples in fp64,
 * centred values rounded to the tensor-core format, zero where unusable or
 * beyond S (padding to Sp columns and Gp rows). */
template <int MODE>
__global__ void k_tc_prep(const float* __restrict__ gem, int G, int S, int Gp, int Sp, float min_expr,
                          void* __restrict__ ops)
{
   const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
   const int lane = threadIdx.x & 31;
   if ( warp >= Gp ) return;
   const size_t plane = (size_t)Gp * Sp;
   double sum = 0.0;
   int n = 0;
   if ( warp < G )
   {
      for ( int s = lane; s < S; s += 32 )
      {
         const float v = gem[(size_t)warp * S + s];
         if ( !isnan(v) && !(v < min_expr) )
         {
            sum += v;
            ++n;
         }
      }
   }
   for ( int o = 16; o > 0; o >>= 1 )
   {
      sum += __shfl_xor_sync(0xffffffffu, sum, o);
      n += __shfl_xor_sync(0xffffffffu, n, o);
   }
   const double mean = n > 0 ? sum / n : 0.0;
   /* FP16: the power of two 2^-e with the gene's largest |a| below 2^e, so |a| 2^-e < 1 */
   float scale = 1.f;
   if ( MODE == 4 )
   {
      float amax = 0.f;
      if ( warp < G )
      {
         for ( int s = lane; s < S; s += 32 )
         {
            const float v = gem[(size_t)warp * S + s];
            if ( !isnan(v) && !(v < min_expr) ) amax = fmaxf(amax, fabsf((float)((double)v - mean)));
         }
      }
      for ( int o = 16; o > 0; o >>= 1 ) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
      if ( amax > 0.f )
      {
         int e;
         frexpf(amax, &e);                           /* amax = f 2^e, 0.5 <= f < 1 */
         scale = ldexpf(1.f, -e);
      }
   }
   for ( int s = lane; s < Sp; s += 32 )
   {
      float a = 0.f, m = 0.f;
      if ( warp < G && s < S )
      {
         const float v = gem[(size_t)warp * S + s];
         if ( !isnan(v) && !(v < min_expr) )
         {
            a = (float)((double)v - mean) * scale;   /* exact: scale is a power of two */
            m = 1.f;
         }
      }
      const float a2 = a * a;
      const size_t o = (size_t)warp * Sp + s;
      if ( MODE == 3 )
      {
         float* f = (float*)ops;
         f[o] = a;
         f[plane + o] = a2;
         f[2 * plane + o] = m;
      }
      else if ( MODE == 4 )
      {
         __half* h = (__half*)ops;
         h[o] = __float2half_rn(a);
         h[plane + o] = __float2half_rn(a2);
         h[2 * plane + o] = __float2half_rn(m);
      }
      else if ( MODE == 1 )
      {
         float* f = (float*)ops;
         uint32_t t;
         asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(t) : "f"(a));
         f[o] = __uint_as_float(t);
         asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(t) : "f"(a2));
         f[plane + o] = __uint_as_float(t);
         f[2 * plane + o] = m;
      }
      else
      {
         __nv_bfloat16* h = (__nv_bfloat16*)ops;
         const __nv_bfloat16 ahi = __float2bfloat16_rn(a);
         const __nv_bfloat16 alo = __float2bfloat16_rn(a - __bfloat162float(ahi));
         const __nv_bfloat16 qhi = __float2bfloat16_rn(a2);
         const __nv_bfloat16 qlo = __float2bfloat16_rn(a2 - __bfloat162float(qhi));
         h[o] = ahi;
         h[plane + o] = alo;
         h[2 * plane + o] = qhi;
         h[3 * plane + o] = qlo;
         h[4 * plane + o] = __float2bfloat16_rn(m);
      }
   }
}

struct TcArgs
{
   int I0;                            /* CUDA-core form: first row tile (blockIdx.y = I - I0, blockIdx.x = J) */
   int64_t xb;                        /* last row of the pair range */
   int G;
   int min_samples;
   int max_k;
   int64_t start, end;                /* pairs written: [start, end) */
   float* out_corr;                   /* [p - start][max_k], column 0 */
   int* status;
   int kchunks;
};

/* error-compensated a*b - c*d in fp32 (the products' rounding errors recovered by fma) */
__device__ __forceinline__ float diff_of_products(float a, float b, float c, float d)
{
   const float cd = c * d;
   const float err = fmaf(-c, d, cd);
   const float dop = fmaf(a, b, -cd);
   return dop + err;
}

/* MMAs of one K-chunk in ring stage `stage` (see the TF32 / 3xBF16 notes above); acc0: 0 on the
 * tile's first chunk (the accumulators start from zero) */
template <int MODE>
__device__ __forceinline__ void issue_chunk(uint32_t tmem, uint32_t stage, bool first)
{
   using C = Cfg<MODE>;
   using L = Layout<MODE>;
   constexpr int BN = C::BN;
   const uint32_t ysb = stage + C::NMAT * L::XMAT;
#pragma unroll
   for ( int ks = 0; ks < C::BK / C::UMMA_K; ++ks )
   {
      const uint32_t koff = ks * C::UMMA_K * C::ELEM;   /* byte step along K inside the row */
      const uint32_t acc = (!first || ks > 0) ? 1u : 0u;
      if ( merged<MODE>() && MODE == 2 )
      {
         /* x side: 0 Ah, 1 Al, 2 Qh, 3 Ql, 4 M; y side in slots [Ql][Qh][Ah][M][Al] */
         const uint64_t xah = smem_desc<MODE>(stage + 0 * L::XMAT + koff);
         const uint64_t xal = smem_desc<MODE>(stage + 1 * L::XMAT + koff);
         const uint64_t xqh = smem_desc<MODE>(stage + 2 * L::XMAT + koff);
         const uint64_t xql = smem_desc<MODE>(stage + 3 * L::XMAT + koff);
         const uint64_t xm = smem_desc<MODE>(stage + 4 * L::XMAT + koff);
         const uint64_t y_ql = smem_desc<MODE>(ysb + 0 * L::YMAT + koff);
         const uint64_t y_qh_ah_m = smem_desc<MODE>(ysb + 1 * L::YMAT + koff);
         const uint64_t y_ah_m_al = smem_desc<MODE>(ysb + 2 * L::YMAT + koff);
         const uint64_t y_m = smem_desc<MODE>(ysb + 3 * L::YMAT + koff);
         const uint64_t y_al = smem_desc<MODE>(ysb + 4 * L::YMAT + koff);
         mma<MODE, 3 * BN>(tmem + 0, xah, y_ah_m_al, acc);      /* Sxy(hh) | Sx(h) | Sxy(hl) */
         mma<MODE, 2 * BN>(tmem + 0, xal, y_ah_m_al, 1u);       /* += Sxy(lh) | Sx(l) */
         mma<MODE, BN>(tmem + acc_col<MODE>(3), xqh, y_m, acc); /* Sxx */
         mma<MODE, BN>(tmem + acc_col<MODE>(3), xql, y_m, 1u);
         mma<MODE, 3 * BN>(tmem + acc_col<MODE>(4), xm, y_qh_ah_m, acc);   /* Syy(h) | Sy(h) | n */
         mma<MODE, BN>(tmem + acc_col<MODE>(4), xm, y_ql, 1u);             /* Syy += l */
         mma<MODE, BN>(tmem + acc_col<MODE>(2), xm, y_al, 1u);             /* Sy += l */
      }
      else if ( merged<MODE>() )
      {
         const uint64_t xa = smem_desc<MODE>(stage + 0 * L::XMAT + koff);
         const uint64_t xq = smem_desc<MODE>(stage + 1 * L::XMAT + koff);
         const uint64_t xm = smem_desc<MODE>(stage + 2 * L::XMAT + koff);
         const uint64_t y_q_a_m = smem_desc<MODE>(ysb + 0 * L::YMAT + koff);   /* [A2_y; A_y; M_y] */
         const uint64_t y_a_m = smem_desc<MODE>(ysb + 1 * L::YMAT + koff);     /* [A_y; M_y] */
         const uint64_t y_m = smem_desc<MODE>(ysb + 2 * L::YMAT + koff);       /* M_y */
         mma<MODE, 2 * BN>(tmem + acc_col<MODE>(0), xa, y_a_m, acc);     /* Sxy | Sx */
         mma<MODE, BN>(tmem + acc_col<MODE>(3), xq, y_m, acc);           /* Sxx */
         mma<MODE, 3 * BN>(tmem + acc_col<MODE>(4), xm, y_q_a_m, acc);   /* Syy | Sy | n */
      }
      else if ( MODE != 2 )
      {
         /* x side: 0 A, 1 A2, 2 M; y side likewise */
         const uint64_t xa = smem_desc<MODE>(stage + 0 * L::XMAT + koff);
         const uint64_t xq = smem_desc<MODE>(stage + 1 * L::XMAT + koff);
         const uint64_t xm = smem_desc<MODE>(stage + 2 * L::XMAT + koff);
         const uint64_t ya = smem_desc<MODE>(ysb + 0 * L::YMAT + koff);
         const uint64_t yq = smem_desc<MODE>(ysb + 1 * L::YMAT + koff);
         const uint64_t ym = smem_desc<MODE>(ysb + 2 * L::YMAT + koff);
         mma<MODE>(tmem + 0 * BN, xa, ya, acc);   /* Sxy */
         mma<MODE>(tmem + 1 * BN, xa, ym, acc);   /* Sx */
         mma<MODE>(tmem + 2 * BN, xm, ya, acc);   /* Sy */
         mma<MODE>(tmem + 3 * BN, xq, ym, acc);   /* Sxx */
         mma<MODE>(tmem + 4 * BN, xm, yq, acc);   /* Syy */
         mma<MODE>(tmem + 5 * BN, xm, ym, acc);   /* n */
      }
      else
      {
         /* 0 A_hi, 1 A_lo, 2 A2_hi, 3 A2_lo, 4 M */
         uint64_t xd[5], yd[5];
#pragma unroll
         for ( int m = 0; m < 5; ++m )
         {
            xd[m] = smem_desc<MODE>(stage + m * L::XMAT + koff);
            yd[m] = smem_desc<MODE>(ysb + m * L::YMAT + koff);
         }
         mma<MODE>(tmem + 0 * BN, xd[0], yd[0], acc);   /* Sxy: hi.hi + hi.lo + lo.hi */
         mma<MODE>(tmem + 0 * BN, xd[0], yd[1], 1u);
         mma<MODE>(tmem + 0 * BN, xd[1], yd[0], 1u);
         mma<MODE>(tmem + 1 * BN, xd[0], yd[4], acc);   /* Sx */
         mma<MODE>(tmem + 1 * BN, xd[1], yd[4], 1u);
         mma<MODE>(tmem + 2 * BN, xd[4], yd[0], acc);   /* Sy */
         mma<MODE>(tmem + 2 * BN, xd[4], yd[1], 1u);
         mma<MODE>(tmem + 3 * BN, xd[2], yd[4], acc);   /* Sxx */
         mma<MODE>(tmem + 3 * BN, xd[3], yd[4], 1u);
         mma<MODE>(tmem + 4 * BN, xd[4], yd[2], acc);   /* Syy */
         mma<MODE>(tmem + 4 * BN, xd[4], yd[3], 1u);
         mma<MODE>(tmem + 5 * BN, xd[4], yd[4], acc);   /* n */
      }
   }
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
   asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

/*
 * Persistent form: one CTA per SM walks its share of the tile list (tile t = blockIdx.x,
 * blockIdx.x + gridDim.x, ...; the host orders the list in bands of TILE_GROUP row tiles, column
 * by column, so the CTAs running at one time share their x- and y-side operand panels in L2).
 * Warp 0 streams the K-chunks of its tiles through the ring without stopping at tile boundaries;
 * warp 1 issues a tile's MMAs once the epilogue has released TMEM from the previous tile and
 * signals `tfull` when the accumulators are final; warps 2..9 (two per TMEM lane quarter, each
 * half of the 64 columns) read them back, form r, signal `tempty` and then write r.  So the next
 * tile's operand loads overlap this tile's epilogue, its MMAs overlap the epilogue's writes, and
 * TMEM, barriers and the ring are set up once per CTA.  Every mbarrier wait is bounded: on expiry the CTA records an error, every role
 * stops, the CTA drains its own copies (bounded), frees its TMEM and returns.
 */

template <int MODE>
__global__ void __launch_bounds__(TC_THREADS, 1)
   k_pearson_tc(const __grid_constant__ TcMaps maps, TcArgs args, const int2* __restrict__ tiles, int ntiles)
{
   using C = Cfg<MODE>;
   using L = Layout<MODE>;
   constexpr int BN = C::BN;
   constexpr int STAGES = C::STAGES;
   extern __shared__ __align__(1024) unsigned char smem_raw[];
   unsigned char* ring = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
   uint64_t* bars = (uint64_t*)(ring + L::RING);
   uint32_t* tmem_holder = (uint32_t*)(bars + 2 * STAGES + 2);
   __shared__ int s_fail;

   /* a CTA that failed earlier in this launch stops the rest from starting (decided once, for
    * the whole CTA) */
   if ( threadIdx.x == 0 ) s_fail = *(volatile int*)args.status != 0;
   __syncthreads();
   if ( s_fail ) return;
   const int warp = threadIdx.x >> 5;
   const int lane = threadIdx.x & 31;
   const uint32_t full0 = smem_u32(&bars[0]);
   const uint32_t empty0 = smem_u32(&bars[STAGES]);
   const uint32_t tfull = smem_u32(&bars[2 * STAGES]);
   const uint32_t tempty = smem_u32(&bars[2 * STAGES + 1]);

   __syncthreads();                     /* every thread has read s_fail before it is reused */
   if ( threadIdx.x == 0 )
   {
      s_fail = 0;
      for ( int s = 0; s < STAGES; ++s )
      {
         mbar_init(full0 + 8 * s, 1);
         mbar_init(empty0 + 8 * s, 1);
      }
      mbar_init(tfull, 1);
      mbar_init(tempty, EPI_WARPS);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
   }
   if ( warp == 1 )
   {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_holder)),
                   "r"(TMEM_COLS));
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
   }
   asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
   __syncthreads();
   asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
   const uint32_t tmem = *tmem_holder;

   const int K = args.kchunks;
   int issued = 0;                      /* producer: TMA chunks issued */
   if ( warp == 0 )
   {
      if ( lane == 0 )
      {
         /* ---- producer: the chunks of every tile of this CTA, back to back */
         for ( int t = blockIdx.x; t < ntiles && !*(volatile int*)&s_fail; t += gridDim.x )
         {
            const int2 ij = tiles[t];
            for ( int kc = 0; kc < K; ++kc, ++issued )
            {
               const int s = issued % STAGES;
               if ( issued >= STAGES && !mbar_wait(empty0 + 8 * s, ((issued / STAGES) - 1) & 1) )
               {
                  atomicExch(&s_fail, 1);
                  break;
               }
               if ( *(volatile int*)&s_fail ) break;
               const uint32_t stage = smem_u32(ring + s * L::STAGE);
               mbar_expect_tx(full0 + 8 * s, L::STAGE);
               for ( int m = 0; m < C::NMAT; ++m )
               {
                  tma_load_2d(stage + m * L::XMAT, &maps.x[m], kc * C::BK, ij.x * BM, full0 + 8 * s);
                  tma_load_2d(stage + C::NMAT * L::XMAT + yslot<MODE>(m) * L::YMAT, &maps.y[m], kc * C::BK,
                              ij.y * BN, full0 + 8 * s);
               }
            }
         }
      }
   }
   else if ( warp == 1 )
   {
      if ( lane == 0 )
      {
         /* ---- MMA issuer */
         int used = 0, tl = 0;
         for ( int t = blockIdx.x; t < ntiles && !*(volatile int*)&s_fail; t += gridDim.x, ++tl )
         {
            if ( tl > 0 && !mbar_wait(tempty, (tl - 1) & 1) )
            {
               atomicExch(&s_fail, 1);
               break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            bool ok = true;
            for ( int kc = 0; kc < K; ++kc, ++used )
            {
               const int s = used % STAGES;
               if ( !mbar_wait(full0 + 8 * s, (used / STAGES) & 1) )
               {
                  ok = false;
                  break;
               }
               asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
               issue_chunk<MODE>(tmem, smem_u32(ring + s * L::STAGE), kc == 0);
               mma_commit(empty0 + 8 * s);      /* frees the stage when these MMAs have read it */
            }
            if ( !ok )
            {
               atomicExch(&s_fail, 1);
               break;
            }
            mma_commit(tfull);                  /* the tile's accumulators are final */
         }
      }
   }
   else
   {
      /* ---- epilogue: warp w reads TMEM lanes 32 (w % 4) .. (its quarter of the tile's rows) and
       * half h = (w - 2) / 4 of the tile's four 16-column chunks.  It forms r for its 32 x 32
       * pairs, hands TMEM back to the MMA warp, and only then writes them: the writes overlap the
       * next tile's MMAs instead of holding them up. */
      const int quarter = warp & 3;
      const int half = (warp - 2) >> 2;
      constexpr int WCH = BN / 32;                 /* 16-column chunks per warp */
      static_assert(BN % 32 == 0, "two warps share a quarter's columns");
      const int c0 = half * WCH;
      float* ebuf = (float*)(ring + L::RING + 256) + (warp - 2) * (32 * 8);
      int tl = 0;
      for ( int t = blockIdx.x; t < ntiles; t += gridDim.x, ++tl )
      {
         /* one lane waits and the warp follows its verdict, so the warp stays converged for the
          * .sync.aligned TMEM loads */
         int go = 0;
         if ( lane == 0 ) go = !*(volatile int*)&s_fail && mbar_wait(tfull, tl & 1);
         go = __shfl_sync(0xffffffffu, go, 0);
         if ( !go )
         {
            if ( lane == 0 ) atomicExch(&s_fail, 1);
            break;
         }
         asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
         const int2 ij = tiles[t];
         const uint32_t lane_base = tmem + ((uint32_t)(quarter * 32) << 16);
         /* r of this lane's row (TMEM lane = pair row) and the warp's columns */
         float r[WCH][16];
         {
#pragma unroll
            for ( int w = 0; w < WCH; ++w )
            {
               const int c = c0 + w;
               /* all of the chunk's accumulators in flight at once, then one wait */
               uint32_t v[NACC + 1][16];
#pragma unroll
               for ( int a = 0; a < NACC; ++a ) tmem_ld16_async(lane_base + acc_col<MODE>(a) + c * 16, v[a]);
               if constexpr ( sxy2_col<MODE>() >= 0 )
                  tmem_ld16_async(lane_base + (uint32_t)sxy2_col<MODE>() + c * 16, v[NACC]);
               tmem_wait_ld();
#pragma unroll
               for ( int jj = 0; jj < 16; ++jj )
               {
                  float sxy = __uint_as_float(v[0][jj]);
                  if constexpr ( sxy2_col<MODE>() >= 0 ) sxy += __uint_as_float(v[NACC][jj]);
                  const float sx = __uint_as_float(v[1][jj]), sy = __uint_as_float(v[2][jj]);
                  const float sxx = __uint_as_float(v[3][jj]), syy = __uint_as_float(v[4][jj]);
                  const float n = __uint_as_float(v[5][jj]);
                  r[w][jj] = __int_as_float(0x7fc00000);
                  if ( n >= (float)args.min_samples && n > 0.f )
                  {
                     const float num = diff_of_products(n, sxy, sx, sy);
                     const float dx = diff_of_products(n, sxx, sx, sx);
                     const float dy = diff_of_products(n, syy, sy, sy);
                     r[w][jj] = num * rsqrtf(dx) * rsqrtf(dy);
                  }
               }
            }
         }
         /* every TMEM read of this warp is complete (tmem_wait_ld): hand TMEM back */
         asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
         __syncwarp();
         if ( lane == 0 ) mbar_arrive(tempty);
         /* written through a 32 x 8 shared-memory tile so that each store covers 8 neighbouring
          * pairs of 4 rows (a lane's own row would put the warp's 32 stores in 32 rows); element
          * (row, col) sits at row * 8 + (col ^ (row / 4)), conflict-free both ways */
         const int64_t x0 = (int64_t)ij.x * BM + quarter * 32;   /* the warp's first row */
#pragma unroll
         for ( int g = 0; g < 2 * WCH; ++g )
         {
            __syncwarp();
#pragma unroll
            for ( int j = 0; j < 8; ++j ) ebuf[lane * 8 + (j ^ (lane >> 2))] = r[g >> 1][(g & 1) * 8 + j];
            __syncwarp();
#pragma unroll
            for ( int i = 0; i < 8; ++i )
            {
               const int rr = 4 * i + (lane >> 3), cc = lane & 7;
               const int64_t x = x0 + rr;
               const int64_t y = (int64_t)ij.y * BN + c0 * 16 + g * 8 + cc;
               const int64_t p = x * (x - 1) / 2 + y;
               if ( x < args.G && y < x && p >= args.start && p < args.end )
                  args.out_corr[(p - args.start) * args.max_k] = ebuf[rr * 8 + (cc ^ i)];
            }
         }
      }
   }
   __syncwarp();

   /* ---- teardown: on failure drain this CTA's copies (bounded), then free TMEM */
   __syncthreads();
   if ( *(volatile int*)&s_fail )
   {
      if ( threadIdx.x == 0 )
      {
         atomicCAS(args.status, 0, ST_TIMEOUT);
         for ( int g = (issued > STAGES ? issued - STAGES : 0); g < issued; ++g )
         {
            mbar_wait(full0 + 8 * (g % STAGES), (g / STAGES) & 1);
         }
      }
      __syncthreads();
   }
   asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
   __syncthreads();
   asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
   if ( warp == 1 )
   {
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
   }
}

/*
 * The TF32 form on CTA pairs (thread-block clusters of two, tcgen05 cta_group::2).  A pair computes
 * a 256 x 64 tile of pairs with M = 256 MMAs that the even CTA issues: each CTA holds the three
 * x-side operands of its 128 rows and the three y-side operands of its 32 of the tile's 64 genes;
 * an MMA reads A from each CTA's own shared memory and B half from each, and writes each CTA's
 * 128 rows of D into that CTA's TMEM.  On one CTA the K-chunk traffic through shared memory -- TMA
 * writing 72 KB per 32 samples, the MMAs reading 24 KB per 8 -- takes longer than the MMAs
 * themselves (TF32 at M = 128, N = 128 + 64 + 192 per 8 samples); on a pair each SM writes 60 KB
 * and reads 18 KB.
 *
 * D columns of an MMA whose B stacks s y-side operands: the even CTA's 32 genes of each operand,
 * then the odd CTA's, i.e. operand k, tile column j at b + (j / 32) 32 s + 32 k + j % 32.
 *
 * Barriers: the even CTA's full[s] counts the copies of both CTAs (its producer arms it with the
 * bytes of both; the odd CTA's copies signal it across the pair); each MMA commit arrives on
 * empty[s] and, at a tile's end, on tfull in both CTAs; the epilogue warps of both CTAs arrive on
 * the even CTA's tempty (count 16).  Every wait is bounded.  The pair meets at a cluster barrier
 * after setting up and again before leaving; before the second, the even CTA waits for its MMAs
 * to complete and each CTA for the last commits on its own barriers, so neither leaves while the
 * other can still read or write its memory.
 *
 * Measured against the one-CTA form (KINC_TC_PAIR selects it): identical results; in ncu, on one
 * 16.7M-pair launch of the 20,000 x 2,000 matrix, 618 against 601 us, tensor pipe busy 61.6
 * against 59.2 % of the time; timed in a loop over 134M-pair blocks, 4.63 against 4.47 ms.  So
 * the bytes through shared memory are not what holds the one-CTA form back: its MMA warp waits
 * for the next stage's copies, and the pair's waits for the later of two SMs' copies.
 */
namespace pair {
constexpr int BMP = 256;                  /* pair-tile rows, 128 per CTA */
constexpr int BNP = 64;                   /* pair-tile columns */
constexpr int HB = BNP / 2;               /* y-side genes per CTA */
constexpr int STAGES = 3;
constexpr int BK = Cfg<1>::BK;            /* 32 samples: 128-byte rows, SWIZZLE_128B */
constexpr int XMAT = 128 * Cfg<1>::ROWB;  /* one x-side operand chunk, 16 KB */
constexpr int YMAT = HB * Cfg<1>::ROWB;   /* one y-side operand chunk, 4 KB */
constexpr int STAGE = 3 * (XMAT + YMAT);
constexpr int RING = STAGES * STAGE;
constexpr int NBAR = 2 * STAGES + 3;      /* full[], empty[], tfull, tempty, done */
constexpr int SMEM = RING + 1024 /* alignment slack */ + 256 /* barriers */ + Layout<1>::EBUF;
static_assert(SMEM <= 227 * 1024, "ring, barriers and epilogue tiles fit the shared memory of one CTA");
static_assert((NBAR + 1) * 8 <= 256, "barriers and the TMEM address fit their 256 bytes");

/* TMEM column of accumulator a (0 Sxy, 1 Sx, 2 Sy, 3 Sxx, 4 Syy, 5 n) for the tile's columns
 * 32 h .. 32 h + 31: A_x.[A_y; M_y] at 0 (s = 2), A2_x.M_y at 128 (s = 1),
 * M_x.[A2_y; A_y; M_y] at 192 (s = 3) */
__host__ __device__ constexpr int acc_col(int a, int h)
{
   return a == 0 ? 64 * h : a == 1 ? 64 * h + 32 : a == 3 ? 128 + 32 * h
        : a == 4 ? 192 + 96 * h : a == 2 ? 224 + 96 * h : 256 + 96 * h;
}

/* the pair MMAs of one K-chunk in ring stage `stage`; y-side operands in slots [A2_y][A_y][M_y] */
__device__ __forceinline__ void issue_chunk(uint32_t tmem, uint32_t stage, bool first)
{
   const uint32_t ysb = stage + 3 * XMAT;
#pragma unroll
   for ( int ks = 0; ks < BK / Cfg<1>::UMMA_K; ++ks )
   {
      const uint32_t koff = ks * Cfg<1>::UMMA_K * Cfg<1>::ELEM;
      const uint32_t acc = (!first || ks > 0) ? 1u : 0u;
      const uint64_t xa = smem_desc<1>(stage + 0 * XMAT + koff);
      const uint64_t xq = smem_desc<1>(stage + 1 * XMAT + koff);
      const uint64_t xm = smem_desc<1>(stage + 2 * XMAT + koff);
      const uint64_t y_q_a_m = smem_desc<1>(ysb + 0 * YMAT + koff);
      const uint64_t y_a_m = smem_desc<1>(ysb + 1 * YMAT + koff);
      const uint64_t y_m = smem_desc<1>(ysb + 2 * YMAT + koff);
      mma_pair_tf32<2 * BNP>(tmem + 0, xa, y_a_m, acc);     /* Sxy | Sx */
      mma_pair_tf32<BNP>(tmem + 128, xq, y_m, acc);         /* Sxx */
      mma_pair_tf32<3 * BNP>(tmem + 192, xm, y_q_a_m, acc); /* Syy | Sy | n */
   }
}
}  // namespace pair

__global__ void __launch_bounds__(TC_THREADS, 1)
   k_pearson_tc2(const __grid_constant__ TcMaps maps, TcArgs args, const int2* __restrict__ tiles, int ntiles)
{
   using namespace pair;
   constexpr int S = STAGES;
   extern __shared__ __align__(1024) unsigned char smem_raw[];
   unsigned char* ring = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
   uint64_t* bars = (uint64_t*)(ring + RING);
   uint32_t* tmem_holder = (uint32_t*)(bars + NBAR);
   __shared__ int s_fail;
   const int rank = (int)cluster_rank();
   const bool lead = rank == 0;
   const int unit0 = blockIdx.x >> 1, ustep = gridDim.x >> 1;
   const int warp = threadIdx.x >> 5;
   const int lane = threadIdx.x & 31;
   const uint32_t full0 = smem_u32(&bars[0]);
   const uint32_t empty0 = smem_u32(&bars[S]);
   const uint32_t tfull = smem_u32(&bars[2 * S]);
   const uint32_t tempty = smem_u32(&bars[2 * S + 1]);
   const uint32_t done = smem_u32(&bars[2 * S + 2]);
   const uint32_t full0_lead = mapa_rank(full0, 0);
   const uint32_t tempty_lead = mapa_rank(tempty, 0);

   if ( threadIdx.x == 0 )
   {
      s_fail = 0;
      for ( int s = 0; s < S; ++s )
      {
         mbar_init(full0 + 8 * s, 1);
         mbar_init(empty0 + 8 * s, 1);
      }
      mbar_init(tfull, 1);
      mbar_init(tempty, 2 * EPI_WARPS);
      mbar_init(done, 1);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
   }
   if ( warp == 1 )
   {
      /* one warp of each CTA: the pair's TMEM, the same columns in both */
      asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_holder)),
                   "r"(TMEM_COLS));
   }
   asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
   __syncthreads();
   cluster_sync();                      /* both CTAs' barriers are initialised before either signals the other */
   asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
   const uint32_t tmem = *tmem_holder;

   const int K = args.kchunks;
   int issued = 0;                      /* producer: K-chunks whose copies this CTA issued */
   if ( warp == 0 )
   {
      if ( lane == 0 )
      {
         /* ---- producer (both CTAs): this CTA's rows and genes of every chunk of the pair's tiles */
         for ( int u = unit0; u < ntiles && !*(volatile int*)&s_fail; u += ustep )
         {
            const int2 ij = tiles[u];
            for ( int kc = 0; kc < K; ++kc, ++issued )
            {
               const int s = issued % S;
               if ( issued >= S && !mbar_wait(empty0 + 8 * s, ((issued / S) - 1) & 1) )
               {
                  atomicExch(&s_fail, 1);
                  break;
               }
               if ( *(volatile int*)&s_fail ) break;
               const uint32_t stage = smem_u32(ring + s * STAGE);
               if ( lead ) mbar_expect_tx(full0 + 8 * s, 2 * STAGE);
               for ( int m = 0; m < 3; ++m )
               {
                  tma_load_2d_pair(stage + m * XMAT, &maps.x[m], kc * BK, ij.x * BMP + rank * BM, full0_lead + 8 * s);
                  tma_load_2d_pair(stage + 3 * XMAT + yslot<1>(m) * YMAT, &maps.y2[m], kc * BK, ij.y * BNP + rank * HB,
                                   full0_lead + 8 * s);
               }
            }
         }
         /* the even CTA's last commits on this CTA's stages have landed */
         if ( !*(volatile int*)&s_fail )
         {
            for ( int g = (issued > S ? issued - S : 0); g < issued; ++g )
            {
               if ( !mbar_wait(empty0 + 8 * (g % S), (g / S) & 1) )
               {
                  atomicExch(&s_fail, 1);
                  break;
               }
            }
         }
      }
   }
   else if ( warp == 1 )
   {
      if ( lead && lane == 0 )
      {
         /* ---- MMA issuer (the even CTA) */
         int used = 0, tl = 0;
         for ( int u = unit0; u < ntiles && !*(volatile int*)&s_fail; u += ustep, ++tl )
         {
            if ( tl > 0 && !mbar_wait_cluster(tempty, (tl - 1) & 1) )
            {
               atomicExch(&s_fail, 1);
               break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            bool ok = true;
            for ( int kc = 0; kc < K; ++kc, ++used )
            {
               const int s = used % S;
               if ( !mbar_wait(full0 + 8 * s, (used / S) & 1) )
               {
                  ok = false;
                  break;
               }
               asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
               pair::issue_chunk(tmem, smem_u32(ring + s * STAGE), kc == 0);
               commit_pair(empty0 + 8 * s, (uint16_t)0x3);   /* frees the stage in both CTAs */
            }
            if ( !ok )
            {
               atomicExch(&s_fail, 1);
               break;
            }
            commit_pair(tfull, (uint16_t)0x3);               /* the tile's accumulators are final */
         }
         /* every MMA issued, reading both CTAs' shared memory, has completed */
         commit_pair(done, (uint16_t)0x1);
         if ( !mbar_wait(done, 0) ) atomicExch(&s_fail, 1);
      }
   }
   else
   {
      /* ---- epilogue (both CTAs): warp w reads TMEM lanes 32 (w % 4) .. -- its quarter of this
       * CTA's 128 rows -- and the tile's columns 32 h .. 32 h + 31, h = (w - 2) / 4 */
      const int quarter = warp & 3;
      const int h = (warp - 2) >> 2;
      float* ebuf = (float*)(ring + RING + 256) + (warp - 2) * (32 * 8);
      int tl = 0;
      for ( int u = unit0; u < ntiles; u += ustep, ++tl )
      {
         int go = 0;
         if ( lane == 0 ) go = !*(volatile int*)&s_fail && mbar_wait(tfull, tl & 1);
         go = __shfl_sync(0xffffffffu, go, 0);
         if ( !go )
         {
            if ( lane == 0 ) atomicExch(&s_fail, 1);
            break;
         }
         asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
         const int2 ij = tiles[u];
         const uint32_t lane_base = tmem + ((uint32_t)(quarter * 32) << 16);
         float r[2][16];
#pragma unroll
         for ( int w = 0; w < 2; ++w )
         {
            uint32_t v[NACC][16];
#pragma unroll
            for ( int a = 0; a < NACC; ++a ) tmem_ld16_async(lane_base + (uint32_t)acc_col(a, h) + w * 16, v[a]);
            tmem_wait_ld();
#pragma unroll
            for ( int jj = 0; jj < 16; ++jj )
            {
               const float sxy = __uint_as_float(v[0][jj]), sx = __uint_as_float(v[1][jj]);
               const float sy = __uint_as_float(v[2][jj]), sxx = __uint_as_float(v[3][jj]);
               const float syy = __uint_as_float(v[4][jj]), n = __uint_as_float(v[5][jj]);
               r[w][jj] = __int_as_float(0x7fc00000);
               if ( n >= (float)args.min_samples && n > 0.f )
               {
                  const float num = diff_of_products(n, sxy, sx, sy);
                  const float dx = diff_of_products(n, sxx, sx, sx);
                  const float dy = diff_of_products(n, syy, sy, sy);
                  r[w][jj] = num * rsqrtf(dx) * rsqrtf(dy);
               }
            }
         }
         /* every TMEM read of this warp is complete (tmem_wait_ld): hand TMEM back */
         asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
         __syncwarp();
         if ( lane == 0 ) mbar_arrive_cluster(tempty_lead);
         /* written through the warp's 32 x 8 shared-memory tile, as in the one-CTA form */
         const int64_t x0 = (int64_t)ij.x * BMP + rank * BM + quarter * 32;
#pragma unroll
         for ( int g = 0; g < 4; ++g )
         {
            __syncwarp();
#pragma unroll
            for ( int j = 0; j < 8; ++j ) ebuf[lane * 8 + (j ^ (lane >> 2))] = r[g >> 1][(g & 1) * 8 + j];
            __syncwarp();
#pragma unroll
            for ( int i = 0; i < 8; ++i )
            {
               const int rr = 4 * i + (lane >> 3), cc = lane & 7;
               const int64_t x = x0 + rr;
               const int64_t y = (int64_t)ij.y * BNP + h * HB + g * 8 + cc;
               const int64_t p = x * (x - 1) / 2 + y;
               if ( x < args.G && y < x && p >= args.start && p < args.end )
                  args.out_corr[(p - args.start) * args.max_k] = ebuf[rr * 8 + (cc ^ i)];
            }
         }
      }
   }
   __syncwarp();

   /* ---- teardown: on failure drain the pair's copies (bounded), then meet, then free TMEM */
   __syncthreads();
   if ( *(volatile int*)&s_fail )
   {
      if ( threadIdx.x == 0 )
      {
         atomicCAS(args.status, 0, ST_TIMEOUT);
         /* the even CTA's full barriers count both CTAs' copies */
         if ( lead )
            for ( int g = (issued > S ? issued - S : 0); g < issued; ++g ) mbar_wait(full0 + 8 * (g % S), (g / S) & 1);
      }
      __syncthreads();
   }
   asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
   __syncthreads();
   cluster_sync();                      /* neither CTA leaves while the other may use its memory */
   asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
   if ( warp == 1 )
   {
      asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
   }
}

/*
 * The dense tcgen05 MMA rate of one operand type (MODE 1 TF32, 2 BF16) with nothing else in the
 * way: one CTA per SM, operands resident in shared memory, one thread issuing M = 128, N = 256 MMAs
 * (4 K-steps of a 128-byte-swizzled chunk) back to back into TMEM, then one commit and a bounded
 * wait.  The ceiling the tensor-core Pearson form is measured against (the library GEMM rate
 * includes its memory traffic).
 */
/* K-major, 128-byte swizzled rows in 8-row atoms (1,024-byte stride): the probe's operand layout */
__device__ __forceinline__ uint64_t peak_desc(uint32_t addr)
{
   uint64_t d = 0;
   d |= (uint64_t)((addr >> 4) & 0x3fff);
   d |= (uint64_t)((1024 >> 4) & 0x3fff) << 32;
   d |= (uint64_t)1 << 46;
   d |= (uint64_t)2 << 61;
   return d;
}

template <int MODE>
__global__ void __launch_bounds__(128, 1) k_tensor_peak(int iters, int* status)
{
   extern __shared__ __align__(1024) unsigned char smem_raw[];
   unsigned char* ops = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
   __shared__ uint64_t bar;
   __shared__ uint32_t holder;
   constexpr int A_BYTES = BM * 128, B_BYTES = 256 * 128;
   for ( int i = threadIdx.x; i < (A_BYTES + B_BYTES) / 4; i += blockDim.x )
      ((uint32_t*)ops)[i] = 0x3f800000u ^ ((uint32_t)i * 2654435761u & 0x007fffffu);   /* values in [1, 2) */
   if ( threadIdx.x == 0 )
   {
      mbar_init(smem_u32(&bar), 1);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
   }
   if ( threadIdx.x < 32 )
   {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&holder)),
                   "r"(TMEM_COLS));
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
   }
   asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   /* the operands, to the tensor core */
   asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
   __syncthreads();
   asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
   const uint32_t tmem = holder;
   if ( threadIdx.x == 0 )
   {
      const uint32_t a = smem_u32(ops), b = smem_u32(ops + A_BYTES);
      for ( int it = 0; it < iters; ++it )
         for ( int ks = 0; ks < 4; ++ks )
            mma<MODE, 256>(tmem, peak_desc(a + ks * 32), peak_desc(b + ks * 32), (it | ks) ? 1u : 0u);
      mma_commit(smem_u32(&bar));
      if ( !mbar_wait(smem_u32(&bar), 0) ) atomicExch(status, ST_TIMEOUT);
   }
   asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
   __syncthreads();
   asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
   if ( threadIdx.x < 32 )
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
}

/*
 * The same contraction on the CUDA cores in FP32 (precision 3): the comparator
 * for the tensor-core forms.  A CTA of 256 threads computes a 64 x 64 tile of
 * pairs; each thread a 4 x 4 block with the six sums in registers (96 FFMA
 * per sample, fed by six 128-bit shared-memory reads).  The operand chunks
 * (3 planes x 32 samples x 64 genes per side) are staged transposed in shared
 * memory -- [plane][sample][gene], so a thread's four genes are one float4 --
 * double-buffered through registers: the next chunk is read from global
 * memory while the current one is multiplied.
 */
constexpr int SB = 64;                /* genes per tile side */
constexpr int SK = 32;                /* samples per chunk */
constexpr int STHREADS = 256;
constexpr int SIMT_SMEM = 2 * 2 * 3 * SK * SB * (int)sizeof(float);   /* two stages, two sides, three planes */

__global__ void __launch_bounds__(STHREADS, 1) k_pearson_simt(const float* __restrict__ ops, int Gp, int Sp,
                                                             TcArgs args)
{
   extern __shared__ __align__(16) float sm[];
   const int I = args.I0 + (int)blockIdx.y;
   const int J = (int)blockIdx.x;
   const int64_t rowmax = (int64_t)(I + 1) * SB - 1;
   const int64_t xmax = rowmax < args.xb ? rowmax : args.xb;
   if ( (int64_t)J * SB >= xmax ) return;    /* no pair x > y in this tile */
   const int t = threadIdx.x;
   const int tx = t & 15, ty = t >> 4;       /* this thread's genes: x rows 4tx.., y rows 4ty.. */
   const int lr = t & 31, lg = t >> 5;       /* loader: rows lr and lr + 32, samples 4lg..4lg+3 */
   const size_t plane = (size_t)Gp * Sp;
   const float* xsrc = ops + (size_t)I * SB * Sp;
   const float* ysrc = ops + (size_t)J * SB * Sp;

   float4 stage[2][3][2];
   auto fetch = [&](int kc) {
#pragma unroll
      for ( int m = 0; m < 3; ++m )
#pragma unroll
         for ( int h = 0; h < 2; ++h )
         {
            const size_t o = m * plane + (size_t)(lr + 32 * h) * Sp + (size_t)kc * SK + 4 * lg;
            stage[0][m][h] = *reinterpret_cast<const float4*>(xsrc + o);
            stage[1][m][h] = *reinterpret_cast<const float4*>(ysrc + o);
         }
   };
   auto put = [&](int buf) {
#pragma unroll
      for ( int side = 0; side < 2; ++side )
#pragma unroll
         for ( int m = 0; m < 3; ++m )
#pragma unroll
            for ( int h = 0; h < 2; ++h )
            {
               float* d = sm + (((buf * 2 + side) * 3 + m) * SK + 4 * lg) * SB + lr + 32 * h;
               const float4 v = stage[side][m][h];
               d[0 * SB] = v.x;
               d[1 * SB] = v.y;
               d[2 * SB] = v.z;
               d[3 * SB] = v.w;
            }
   };

   float sxy[4][4] = {}, sx[4][4] = {}, sy[4][4] = {}, sxx[4][4] = {}, syy[4][4] = {}, nn[4][4] = {};
   const int K = args.kchunks;
   fetch(0);
   put(0);
   __syncthreads();
   for ( int kc = 0; kc < K; ++kc )
   {
      const int buf = kc & 1;
      if ( kc + 1 < K ) fetch(kc + 1);
      const float* xa = sm + ((buf * 2 + 0) * 3 + 0) * SK * SB + 4 * tx;
      const float* xq = xa + SK * SB;
      const float* xm = xq + SK * SB;
      const float* ya = sm + ((buf * 2 + 1) * 3 + 0) * SK * SB + 4 * ty;
      const float* yq = ya + SK * SB;
      const float* ym = yq + SK * SB;
#pragma unroll 4
      for ( int k = 0; k < SK; ++k )
      {
         const float4 a4 = *reinterpret_cast<const float4*>(xa + k * SB);
         const float4 q4 = *reinterpret_cast<const float4*>(xq + k * SB);
         const float4 m4 = *reinterpret_cast<const float4*>(xm + k * SB);
         const float4 b4 = *reinterpret_cast<const float4*>(ya + k * SB);
         const float4 r4 = *reinterpret_cast<const float4*>(yq + k * SB);
         const float4 n4 = *reinterpret_cast<const float4*>(ym + k * SB);
         const float ax[4] = { a4.x, a4.y, a4.z, a4.w }, qx[4] = { q4.x, q4.y, q4.z, q4.w };
         const float mx[4] = { m4.x, m4.y, m4.z, m4.w };
         const float ay[4] = { b4.x, b4.y, b4.z, b4.w }, qy[4] = { r4.x, r4.y, r4.z, r4.w };
         const float my[4] = { n4.x, n4.y, n4.z, n4.w };
#pragma unroll
         for ( int i = 0; i < 4; ++i )
#pragma unroll
            for ( int j = 0; j < 4; ++j )
            {
               sxy[i][j] = fmaf(ax[i], ay[j], sxy[i][j]);
               sx[i][j] = fmaf(ax[i], my[j], sx[i][j]);
               sy[i][j] = fmaf(mx[i], ay[j], sy[i][j]);
               sxx[i][j] = fmaf(qx[i], my[j], sxx[i][j]);
               syy[i][j] = fmaf(mx[i], qy[j], syy[i][j]);
               nn[i][j] = fmaf(mx[i], my[j], nn[i][j]);
            }
      }
      if ( kc + 1 < K )
      {
         put(buf ^ 1);          /* the other buffer: last read before the previous barrier */
         __syncthreads();
      }
   }

#pragma unroll
   for ( int i = 0; i < 4; ++i )
   {
      const int64_t x = (int64_t)I * SB + 4 * tx + i;
      if ( x >= args.G ) continue;
      const int64_t pbase = x * (x - 1) / 2;
#pragma unroll
      for ( int j = 0; j < 4; ++j )
      {
         const int64_t y = (int64_t)J * SB + 4 * ty + j;
         if ( y >= x ) continue;
         const int64_t p = pbase + y;
         if ( p < args.start || p >= args.end ) continue;
         const float n = nn[i][j];
         float r = __int_as_float(0x7fc00000);
         if ( n >= (float)args.min_samples && n > 0.f )
         {
            const float num = diff_of_products(n, sxy[i][j], sx[i][j], sy[i][j]);
            const float dx = diff_of_products(n, sxx[i][j], sx[i][j], sx[i][j]);
            const float dy = diff_of_products(n, syy[i][j], sy[i][j], sy[i][j]);
            r = num * rsqrtf(dx) * rsqrtf(dy);
         }
         args.out_corr[(p - args.start) * args.max_k] = r;
      }
   }
}

/* K = 1 and NaN beyond column 0 for the pairs of the range (clusmethod none) */
__global__ void k_tc_fill(int64_t size, int max_k, int8_t* __restrict__ K, float* __restrict__ corr)
{
   for ( int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < size; t += (int64_t)gridDim.x * blockDim.x )
   {
      if ( K ) K[t] = 1;
      for ( int k = 1; k < max_k; ++k ) corr[t * max_k + k] = __int_as_float(0x7fc00000);
   }
}

/* ---------------------------------------------------------------- host */

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn()
{
   static EncodeTiledFn fn = nullptr;
   if ( !fn )
   {
      void* p = nullptr;
      cudaDriverEntryPointQueryResult q;
      if ( cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess
           && q == cudaDriverEntryPointSuccess )
         fn = (EncodeTiledFn)p;
   }
   return fn;
}

}  // namespace kinc_tc

using namespace kinc_tc;

/* rows of a tensor-core tile: 256 for the CTA-pair TF32 kernel, else 128 */
static int tc_row_tile(int mode)
{
   return (mode == 1 && KINC_TC_PAIR) ? pair::BMP : BM;
}

/* prepare operands and tensor maps; returns a CUDA error or cudaSuccess */
cudaError_t tc_prepare(TcState& t, const float* d_gem, int G, int S, float min_expr, int mode, cudaStream_t st,
                       char* err, size_t errlen)
{
   t.mode = mode;
   const int rows = tc_row_tile(mode);
   t.Gp = (G + rows - 1) / rows * rows;
   t.Sp = (S + 63) / 64 * 64;
   const int elem = (mode == 2 || mode == 4) ? 2 : 4;
   const int nmat = mode == 2 ? 5 : 3;
   const size_t plane = (size_t)t.Gp * t.Sp * elem;
   cudaError_t e = cudaMalloc(&t.ops, plane * nmat);
   if ( e != cudaSuccess ) return e;
   const int blocks = (t.Gp * 32 + 255) / 256;
   if ( mode == 1 )
   {
      k_tc_prep<1><<<blocks, 256, 0, st>>>(d_gem, G, S, t.Gp, t.Sp, min_expr, t.ops);
   }
   else if ( mode == 2 )
   {
      k_tc_prep<2><<<blocks, 256, 0, st>>>(d_gem, G, S, t.Gp, t.Sp, min_expr, t.ops);
   }
   else if ( mode == 4 )
   {
      k_tc_prep<4><<<blocks, 256, 0, st>>>(d_gem, G, S, t.Gp, t.Sp, min_expr, t.ops);
   }
   else
   {
      k_tc_prep<3><<<blocks, 256, 0, st>>>(d_gem, G, S, t.Gp, t.Sp, min_expr, t.ops);
   }
   e = cudaGetLastError();
   if ( e != cudaSuccess ) return e;
   if ( mode == 3 ) return cudaSuccess;      /* the CUDA-core form reads the planes directly */
   EncodeTiledFn enc = encode_fn();
   if ( !enc )
   {
      snprintf(err, errlen, "cuTensorMapEncodeTiled is not available");
      return cudaErrorNotSupported;
   }
   const int bk = mode == 1 ? Cfg<1>::BK : mode == 4 ? Cfg<4>::BK : Cfg<2>::BK;
   const int bn = mode == 1 ? Cfg<1>::BN : mode == 4 ? Cfg<4>::BN : Cfg<2>::BN;
   for ( int m = 0; m < nmat; ++m )
   {
      char* base = (char*)t.ops + m * plane;
      const cuuint64_t dims[2] = { (cuuint64_t)t.Sp, (cuuint64_t)t.Gp };
      const cuuint64_t strides[1] = { (cuuint64_t)t.Sp * elem };
      const cuuint32_t estr[2] = { 1, 1 };
      const CUtensorMapDataType dt = mode == 1   ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                     : mode == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16
                                                 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
      const int rowb = mode == 1 ? Cfg<1>::ROWB : mode == 4 ? Cfg<4>::ROWB : Cfg<2>::ROWB;
      const CUtensorMapSwizzle sw = rowb == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B;
      const cuuint32_t boxx[2] = { (cuuint32_t)bk, (cuuint32_t)BM };
      const cuuint32_t boxy[2] = { (cuuint32_t)bk, (cuuint32_t)bn };
      CUresult r1 = enc(&t.maps.x[m], dt, 2, base, dims, strides, boxx, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, sw,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
      CUresult r2 = enc(&t.maps.y[m], dt, 2, base, dims, strides, boxy, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, sw,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
      CUresult r3 = CUDA_SUCCESS;
      if ( mode == 1 )
      {
         /* the CTA-pair kernel's y-side boxes: each CTA's 32 of a tile's 64 genes */
         const cuuint32_t boxh[2] = { (cuuint32_t)bk, (cuuint32_t)pair::HB };
         r3 = enc(&t.maps.y2[m], dt, 2, base, dims, strides, boxh, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, sw,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
      }
      if ( r1 != CUDA_SUCCESS || r2 != CUDA_SUCCESS || r3 != CUDA_SUCCESS )
      {
         snprintf(err, errlen, "cuTensorMapEncodeTiled failed (%d, %d, %d)", (int)r1, (int)r2, (int)r3);
         return cudaErrorInvalidValue;
      }
   }
   return cudaSuccess;
}

void tc_release(TcState& t)
{
   if ( t.ops ) cudaFree(t.ops);
   t.ops = nullptr;
   if ( t.d_tiles ) cudaFree(t.d_tiles);
   if ( t.h_tiles ) cudaFreeHost(t.h_tiles);
   if ( t.tiles_ev ) cudaEventDestroy(t.tiles_ev);
   t.d_tiles = nullptr;
   t.h_tiles = nullptr;
   t.tiles_ev = nullptr;
   t.tiles_cap = 0;
   t.tiles_ia = t.tiles_ib = -1;
   t.tiles_xb = -1;
}

/*
 * The tensor-core form's tile list for row tiles Ia..Ib (rows up to xb): every 128 x 64 tile
 * (I, J) with a pair y < x, in bands of TILE_GROUP row tiles, column by column within a band and
 * row by row within a column.  The persistent CTAs take the list round robin, so the tiles
 * running at one time lie in one band and a few columns: TILE_GROUP x-side row panels and a few
 * y-side column panels, which stay in L2 while the band's rows reuse them.  Built on the host into
 * pinned memory and copied on the stream; the copy of the previous list must be complete before
 * the host buffer is rewritten.
 */
constexpr int TILE_GROUP = 8;


static cudaError_t tc_tile_list(TcState& t, int Ia, int Ib, int64_t xb, cudaStream_t st)
{
   if ( t.tiles_ia == Ia && t.tiles_ib == Ib && t.tiles_xb == xb ) return cudaSuccess;
   const int bn = t.mode == 1 ? Cfg<1>::BN : t.mode == 4 ? Cfg<4>::BN : Cfg<2>::BN;
   const int bm = tc_row_tile(t.mode);
   const int group = TILE_GROUP * BM / bm;      /* the same 1,024 rows per band */
   auto jhi = [&](int I) {
      const int64_t rowmax = std::min<int64_t>((int64_t)(I + 1) * bm - 1, xb);
      return rowmax >= 1 ? (int)((rowmax - 1) / bn) : -1;   /* last column tile holding some y < x */
   };
   int64_t n = 0;
   for ( int I = Ia; I <= Ib; ++I ) n += jhi(I) + 1;
   if ( n > INT32_MAX ) return cudaErrorInvalidValue;
   cudaError_t e;
   if ( t.tiles_ev )
   {
      e = cudaEventSynchronize(t.tiles_ev);
      if ( e != cudaSuccess ) return e;
   }
   else
   {
      e = cudaEventCreateWithFlags(&t.tiles_ev, cudaEventDisableTiming);
      if ( e != cudaSuccess ) return e;
   }
   if ( n > t.tiles_cap )
   {
      /* the device list may still be read by an earlier launch (on any stream) */
      e = cudaDeviceSynchronize();
      if ( e != cudaSuccess ) return e;
      if ( t.d_tiles ) cudaFree(t.d_tiles);
      if ( t.h_tiles ) cudaFreeHost(t.h_tiles);
      t.d_tiles = nullptr;
      t.h_tiles = nullptr;
      t.tiles_cap = 0;
      e = cudaMalloc(&t.d_tiles, (size_t)n * sizeof(int2));
      if ( e != cudaSuccess ) return e;
      e = cudaMallocHost(&t.h_tiles, (size_t)n * sizeof(int2));
      if ( e != cudaSuccess ) return e;
      t.tiles_cap = n;
   }
   int64_t k = 0;
   for ( int b0 = Ia; b0 <= Ib; b0 += group )
   {
      const int b1 = std::min(Ib, b0 + group - 1);
      for ( int J = 0; J <= jhi(b1); ++J )
         for ( int I = b0; I <= b1; ++I )
            if ( J <= jhi(I) ) t.h_tiles[k++] = make_int2(I, J);
   }
   t.ntiles = (int)k;
   t.tiles_ia = Ia;
   t.tiles_ib = Ib;
   t.tiles_xb = xb;
   if ( k == 0 ) return cudaSuccess;
   e = cudaMemcpyAsync(t.d_tiles, t.h_tiles, (size_t)k * sizeof(int2), cudaMemcpyHostToDevice, st);
   if ( e != cudaSuccess ) return e;
   return cudaEventRecord(t.tiles_ev, st);
}

/* the persistent one-CTA tensor-core kernel over the current tile list, one CTA per SM */
template <int MODE>
static cudaError_t tc_launch(const TcState& t, const TcArgs& a, cudaStream_t st)
{
   const int smem = Layout<MODE>::SMEM;
   cudaError_t e = cudaFuncSetAttribute(k_pearson_tc<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
   if ( e != cudaSuccess ) return e;
   int dev = 0, sms = 0;
   e = cudaGetDevice(&dev);
   if ( e == cudaSuccess ) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
   if ( e != cudaSuccess ) return e;
   const int grid = std::max(1, std::min(sms, t.ntiles));
   k_pearson_tc<MODE><<<grid, TC_THREADS, smem, st>>>(t.maps, a, t.d_tiles, t.ntiles);
   return cudaGetLastError();
}

/* the CTA-pair TF32 kernel: as many pairs as can be resident at once (a pair needs two free SMs
 * of one GPC), each walking the list of 256 x 64 pair tiles */
static cudaError_t tc_launch_pair(const TcState& t, const TcArgs& a, cudaStream_t st)
{
   const int smem = pair::SMEM;
   cudaError_t e = cudaFuncSetAttribute(k_pearson_tc2, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
   if ( e != cudaSuccess ) return e;
   cudaLaunchConfig_t cfg = {};
   cudaLaunchAttribute attr[1];
   cfg.gridDim = dim3(2);
   cfg.blockDim = dim3(TC_THREADS);
   cfg.dynamicSmemBytes = (size_t)smem;
   cfg.stream = st;
   attr[0].id = cudaLaunchAttributeClusterDimension;
   attr[0].val.clusterDim.x = 2;
   attr[0].val.clusterDim.y = 1;
   attr[0].val.clusterDim.z = 1;
   cfg.attrs = attr;
   cfg.numAttrs = 1;
   int resident = 0;
   e = cudaOccupancyMaxActiveClusters(&resident, k_pearson_tc2, &cfg);
   if ( e != cudaSuccess ) return e;
   if ( resident < 1 ) return cudaErrorLaunchOutOfResources;
   cfg.gridDim = dim3((unsigned)(2 * std::max(1, std::min(resident, t.ntiles))));
   return cudaLaunchKernelEx(&cfg, k_pearson_tc2, t.maps, a, (const int2*)t.d_tiles, t.ntiles);
}

/* enqueue the pairs [start, start+size): K = 1, corr[.][0] = r, NaN elsewhere */
cudaError_t tc_enqueue(TcState& t, int G, int S, int min_samples, int max_k, int64_t start, int64_t size,
                       int8_t* d_K, float* d_corr, int* d_status, cudaStream_t st, int* launches)
{
   const int64_t end = start + size;
   /* rows touched by the range */
   auto row_of = [](int64_t p) {
      int64_t x = (int64_t)((1.0 + sqrt(1.0 + 8.0 * (double)p)) * 0.5);
      while ( x * (x - 1) / 2 > p ) --x;
      while ( (x + 1) * x / 2 <= p ) ++x;
      return x;
   };
   const int64_t xa = row_of(start);
   const int64_t xb = row_of(end - 1);
   const int tile_x = t.mode == 3 ? SB : tc_row_tile(t.mode);
   const int tile_y = t.mode == 3 ? SB : t.mode == 1 ? Cfg<1>::BN : t.mode == 4 ? Cfg<4>::BN : Cfg<2>::BN;
   const int Ia = (int)(xa / tile_x), Ib = (int)(xb / tile_x);
   const int Jn = (int)((xb + tile_y - 1) / tile_y);
   if ( Jn < 1 ) return cudaSuccess;
   k_tc_fill<<<(int)std::min<int64_t>((size + 255) / 256, 65535), 256, 0, st>>>(size, max_k, d_K, d_corr);
   TcArgs a;
   a.I0 = Ia;
   a.xb = xb;
   a.G = G;
   a.min_samples = min_samples;
   a.max_k = max_k;
   a.start = start;
   a.end = end;
   a.out_corr = d_corr;
   a.status = d_status;
   a.kchunks = t.Sp / (t.mode == 1 ? Cfg<1>::BK : t.mode == 4 ? Cfg<4>::BK : Cfg<2>::BK);   /* Sp: a multiple of 64 */
   if ( t.mode == 3 )
   {
      a.kchunks = t.Sp / SK;
      cudaFuncSetAttribute(k_pearson_simt, cudaFuncAttributeMaxDynamicSharedMemorySize, SIMT_SMEM);
      k_pearson_simt<<<dim3((unsigned)Jn, (unsigned)(Ib - Ia + 1)), STHREADS, SIMT_SMEM, st>>>(
         (const float*)t.ops, t.Gp, t.Sp, a);
   }
   else
   {
      const cudaError_t e = tc_tile_list(t, Ia, Ib, xb, st);
      if ( e != cudaSuccess ) return e;
      if ( t.ntiles == 0 ) return cudaGetLastError();
      const cudaError_t le = t.mode == 2   ? tc_launch<2>(t, a, st)
                             : t.mode == 4 ? tc_launch<4>(t, a, st)
                             : KINC_TC_PAIR ? tc_launch_pair(t, a, st)
                                            : tc_launch<1>(t, a, st);
      if ( le != cudaSuccess ) return le;
   }
   if ( launches ) *launches += 2;
   (void)S;
   return cudaGetLastError();
}

/* dense tcgen05 MMA rate of the current device for precision 1 (TF32) or 2 (BF16), in TFLOP/s */
extern "C" int kinc_sim_tensor_peak(int32_t precision, double* tflops)
{
   if ( (precision != 1 && precision != 2) || !tflops ) return KINC_SIM_EINVAL;
   int dev = 0, sms = 0;
   if ( cudaGetDevice(&dev) != cudaSuccess ) return KINC_SIM_ECUDA;
   if ( cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ) return KINC_SIM_ECUDA;
   int* d_status = nullptr;
   if ( cudaMalloc(&d_status, sizeof(int)) != cudaSuccess ) return KINC_SIM_ENOMEM;
   cudaEvent_t e0 = nullptr, e1 = nullptr;
   const int smem = 160 * 1024;   /* one CTA per SM */
   const int iters = 20000;
   int rc = KINC_SIM_OK;
   float best = 0.f;
   if ( cudaMemset(d_status, 0, sizeof(int)) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess )
      rc = KINC_SIM_ECUDA;
   if ( rc == KINC_SIM_OK )
   {
      cudaFuncSetAttribute(k_tensor_peak<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
      cudaFuncSetAttribute(k_tensor_peak<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
      for ( int rep = 0; rep < 3 && rc == KINC_SIM_OK; ++rep )
      {
         cudaEventRecord(e0);
         if ( precision == 1 )
            k_tensor_peak<1><<<sms, 128, smem>>>(iters, d_status);
         else
            k_tensor_peak<2><<<sms, 128, smem>>>(iters, d_status);
         cudaEventRecord(e1);
         float ms = 0.f;
         if ( cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess )
            rc = KINC_SIM_ECUDA;
         else if ( rep > 0 && (best == 0.f || ms < best) )
            best = ms;   /* the first launch is the warm-up */
      }
   }
   int st = 0;
   if ( rc == KINC_SIM_OK && cudaMemcpy(&st, d_status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess )
      rc = KINC_SIM_ECUDA;
   if ( rc == KINC_SIM_OK && st != 0 ) rc = KINC_SIM_EKERNEL;
   if ( e0 ) cudaEventDestroy(e0);
   if ( e1 ) cudaEventDestroy(e1);
   cudaFree(d_status);
   if ( rc != KINC_SIM_OK ) return rc;
   const double k = precision == 1 ? 8.0 : 16.0;
   *tflops = 2.0 * BM * 256 * k * 4.0 * iters * sms / (best * 1e-3) / 1e12;
   return KINC_SIM_OK;
}
