/*
 * sim_device.cuh -- device code of the GB300 Similarity worker.
 *
 * Execution model.  One warp owns a tile of 32 gene pairs at a time (a
 * persistent grid takes tiles from a counter in global memory; the pairs of
 * a launch are ordered by usable-sample count, largest first).  Work whose result does
 * not depend on evaluation order -- fetching and compacting the pair,
 * Tukey quartiles (order statistics), the Spearman bitonic network -- runs
 * warp-cooperatively, one pair after another, with the pair's data staged in
 * shared memory.  Work whose result depends on the order of floating-point
 * operations -- every EM / Lloyd / Pearson sum, which the reference
 * accumulates sequentially in sample order -- runs one pair per lane, each
 * lane repeating the reference's exact operation sequence on its own pair.
 * Per-pair arrays live in global scratch interleaved by lane ([i][32]), so
 * lane-parallel passes are coalesced.  The whole translation unit is built
 * with --fmad=false so no a*b+c is contracted; kinc_fmath.h supplies exp/log.
 *
 * Reference semantics restated here (paths relative to the KINC tree):
 *   fetchPair                 src/core/similarity_serial.cpp:108-141
 *   Clustering::compute       src/core/pairwise_clustering.cpp:23-103
 *   markOutliers              src/core/pairwise_clustering.cpp:110-148
 *   computeBIC / computeICL   src/core/pairwise_clustering.cpp:155-172
 *   GMM::fit and helpers      src/core/pairwise_gmm.cpp:11-445
 *   KMeans::fit               src/core/pairwise_kmeans.cpp:12-127
 *   Pearson::computeCluster   src/core/pairwise_pearson.cpp:12-52
 *   Spearman::computeCluster  src/core/pairwise_spearman.cpp:27-166
 */
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "kinc_f2.h"
#include "kinc_fmath.h"

namespace kinc {

/* L2 prefetch of one lane's scratch word; the callers keep the address inside
 * the lane's own [0, N) samples */
__device__ __forceinline__ void prefetch_l2(const void* p)
{
   asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

constexpr int TILE = 32;            /* pairs per warp tile */
#ifndef KINC_SAMPLE_UNROLL
#define KINC_SAMPLE_UNROLL 1
#endif
constexpr int SAMPLE_UNROLL = KINC_SAMPLE_UNROLL;   /* unroll factor of the EM sample loops */
#ifndef KINC_PREFETCH
#define KINC_PREFETCH 8             /* samples ahead the Lloyd sweeps prefetch into L2 (0: none); the EM
                                       sweeps take theirs from DevParams::prefetch */
#endif
#ifndef KINC_KM_RING
#define KINC_KM_RING 2              /* samples the Lloyd sweep keeps in flight in registers */
#endif
constexpr int KM_RING = KINC_KM_RING;
#ifndef KINC_UNROLL_SMALL_K
#define KINC_UNROLL_SMALL_K 0       /* fits with K <= this unroll their sample loops by 2 (more ILP) */
#endif
#ifndef KINC_STATIC_K
#define KINC_STATIC_K 1             /* 1: one compiled fit per K (K known to the compiler); 0: one fit for all K <= KS */
#endif
#ifndef KINC_GMM_PARAMS_SMEM
#define KINC_GMM_PARAMS_SMEM 0      /* 1: GMM component parameters live in shared memory, read per use */
#endif
#ifndef KINC_PARAMS_VOLATILE
#define KINC_PARAMS_VOLATILE 0
#endif
#if KINC_PARAMS_VOLATILE
#define PARAM_QUAL volatile
#else
#define PARAM_QUAL
#endif
/* 1: the E step keeps log(gamma/pi) per sample and component for M1 and the label pass; measured
 * slower (96k vs 130k pairs/s on GMM k <= 5, 5,000 x 1,000): M1's exps then wait on a load per
 * component instead of recomputing the log-density from the sample already in a register */
#ifndef KINC_STORE_LOGGAMMA
#define KINC_STORE_LOGGAMMA 0
#endif
/* 1: GMM fits with K >= 2 pair their components in packed FP32 registers (gmm_fit_packed) */
#ifndef KINC_GMM_PACKED
#define KINC_GMM_PACKED 1
#endif
#ifndef KINC_GMM_M2_UNROLL
#define KINC_GMM_M2_UNROLL 2        /* gmm_fit_packed: unroll of the M2 sample loop (its loads of several samples in
                                       flight; 2: +0.5 %, 4: -0.6 %) */
#endif
#ifndef KINC_GMM_E_UNROLL
#define KINC_GMM_E_UNROLL 1         /* gmm_fit_packed: unroll of the E-step sample loop (2: -3 %) */
#endif
#ifndef KINC_GMM_RING
#define KINC_GMM_RING 1             /* gmm_fit_packed: samples the E and M1 sweeps load ahead into registers (2: -0.7 %) */
#endif
#ifndef KINC_GMM_PIPE_G
#define KINC_GMM_PIPE_G 1           /* 1: gmm_fit's M2 loads the next sample's responsibilities a step ahead */
#endif
#ifndef KINC_STORE_GAMMA
#define KINC_STORE_GAMMA 1          /* 1: keep the M1 responsibilities for M2 instead of recomputing them */
#endif
constexpr int RNG_WORDS = 31;       /* glibc TYPE_3 state words */
constexpr int RNG_BITS = 48;        /* jump table covers positions < 2^48 */

/* status codes a kernel may raise (first one wins) */
constexpr int ST_OK = 0;
constexpr int ST_BAD_RANK = 1;      /* fetched N disagrees with the pre-pass count */

struct DevParams
{
   int32_t G, S, W;                 /* genes, samples, 32-bit mask words per gene */
   int32_t clus, corr;
   float min_expr;
   int32_t min_samples, min_k, max_k, criterion, pre_out, post_out;
   int32_t semantics, rand_mode;
   int64_t draws_per_pair;          /* glibc draws one qualifying pair consumes */
   double c2;                       /* D * log(2 pi), D = 2, in double */
   int32_t P2;                      /* next power of two >= max(S, 2) */
   int32_t sort_floats;             /* floats of sort buffer per warp */
   int32_t gam_k;                   /* components per sample in DevScratch::gam (0: none) */
   int32_t ncorr;                   /* correlations per cluster: 1, or 2 for Pearson and Spearman */
   /* launch shape (results are the same for every choice) */
   int32_t warps;                   /* warps per CTA */
   int32_t rounds;                  /* 1: a CTA's warps take their tiles together, round by round */
   int32_t prefetch;                /* samples ahead the EM sweeps prefetch into L2 (0: none) */
   int32_t km_dmax, km_tmax;        /* K-means task pool: draws per pair, tasks per tile */
   float neg_zero;                  /* -0.0f, a value the compiler cannot see (kinc_f2.h: mulz) */
};

struct DevData
{
   const float* gem;                /* [G][S] */
   const uint32_t* umask;           /* [G][W] usable: !isnan && !(v < minexpr) */
   const double* logn;              /* [S+1] log((double)N) */
   const uint32_t* jump;            /* [RNG_BITS][31][31] A^(2^b), [b][col][row] */
   const uint32_t* rng0;            /* [31] state before output 0 */
};

struct DevScratch
{
   float2* X;                       /* per warp slot: [S][32] */
   float* lpx;                      /* per warp slot: [S][32] */
   float* gam;                      /* per warp slot: [S][gam_k][32] GMM responsibilities */
   int8_t* lbl;                     /* per warp slot: [S][32] */
   int8_t* wl;                      /* per warp slot: [S][32] work labels */
   int8_t* ya;                      /* per warp slot: [S][32] K-means */
   int8_t* yb;
   int8_t* yc;
   uint32_t* rng;                   /* per warp slot: [31][32] */
   float* sortbuf;                  /* per warp slot: sort_floats, used when not in shared memory */
   float2* Xl;                      /* K-means: per lane [S], the lane's samples contiguous */
   int32_t* kmd;                    /* K-means task pool: per warp slot [km_dmax][32] rand() draws */
   float* kmr;                      /* K-means task pool: per warp slot [km_tmax][record floats] */
};

struct DevBlock
{
   int64_t start, size;             /* pairs of this launch */
   int64_t lo;                      /* first pair covered by N[] / pg[] (start of its work block) */
   const int32_t* N;                /* [p - lo] */
   const int32_t* pg;               /* [p - lo]: previous pair in the work block with larger N, or -1 */
   const uint64_t* qpos;            /* [p - start]: qualifying pairs before p (rand position / draws) */
   const int32_t* order;            /* tile slot -> p - start (pairs binned by N, largest first); NULL: identity */
   int8_t* outK;                    /* [p - start] */
   int8_t* outLabels;               /* [p - start][S] */
   float* outCorr;                  /* [p - start][max_k] */
   unsigned long long* tiles;       /* tile queue counter */
   int* status;
   unsigned long long* work;        /* [0] model units: sum over fits of iterations x N x K;
                                       [1] fits run */
};

/* ------------------------------------------------------------- helpers */

__device__ __forceinline__ void pair_xy(int64_t p, int32_t& x, int32_t& y)
{
   /* inverse of p = x(x-1)/2 + y, x > y >= 0 (src/core/pairwise_index.cpp:32-57) */
   /* float estimate (GB300's FP64 rate is a small fraction of FP32), corrected exactly below */
   int64_t xx = (int64_t)((1.0f + sqrtf(1.0f + 8.0f * (float)p)) * 0.5f);
   while ( xx * (xx - 1) / 2 > p ) --xx;
   while ( (xx + 1) * xx / 2 <= p ) ++xx;
   x = (int32_t)xx;
   y = (int32_t)(p - xx * (xx - 1) / 2);
}

__device__ __forceinline__ unsigned lanemask_lt()
{
   unsigned m;
   asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
   return m;
}

__device__ __forceinline__ int next_pow2(int n)
{
   int p = 2;
   while ( p < n ) p *= 2;
   return p;
}

/* Spearman::bitonicSort network (pairwise_spearman.cpp:109-134) executed by a
 * warp: every stage's compare-exchanges touch disjoint slots, so running them
 * in parallel performs exactly the reference's sequence of swaps. */
__device__ inline void warp_bitonic(int size, float* key, float* extra, int lane)
{
   const int bsize = size / 2;
   for ( int ob = 2; ob <= size; ob *= 2 )
   {
      const int half = ob / 2;
      for ( int ib = ob; ib >= 2; ib /= 2 )
      {
         const int t = ib / 2;
         for ( int i = lane; i < bsize; i += 32 )
         {
            const bool desc = (i / half) & 1;
            const int a = (i / t) * ib + (i % t);
            const int b = a + t;
            const float ka = key[a];
            const float kb = key[b];
            if ( (ka > kb && !desc) || (ka < kb && desc) )
            {
               key[a] = kb;
               key[b] = ka;
               if ( extra )
               {
                  const float ea = extra[a];
                  extra[a] = extra[b];
                  extra[b] = ea;
               }
            }
         }
         __syncwarp();
      }
   }
}

/* ----------------------------------------------------------- rand() */

/* glibc rand() from a 31-word lagged-Fibonacci state kept in scratch,
 * interleaved by lane; head = index of the oldest word. */
struct LaneRng
{
   uint32_t* ring;
   int head;
   int mode;
   uint64_t lcg;

   __device__ __forceinline__ int32_t next()
   {
      if ( mode == 0 )
      {
         int h28 = head + 28;
         if ( h28 >= RNG_WORDS ) h28 -= RNG_WORDS;
         const uint32_t v = ring[head * TILE] + ring[h28 * TILE];
         ring[head * TILE] = v;
         head = head + 1 == RNG_WORDS ? 0 : head + 1;
         return (int32_t)(v >> 1);
      }
      lcg = lcg * 1103515245ull + 12345ull;
      return (int32_t)((uint32_t)(lcg / 65536ull) % 32768u);
   }
};

/* The glibc state at output position `pos`, warp-cooperatively: lane r < 31
 * returns word r. */
__device__ inline uint32_t warp_rng_state(const DevData& D, uint64_t pos, int lane)
{
   uint32_t s = lane < RNG_WORDS ? D.rng0[lane] : 0u;
   for ( int b = 0; b < RNG_BITS && pos; ++b, pos >>= 1 )
   {
      if ( !(pos & 1) ) continue;
      const uint32_t* M = D.jump + (size_t)b * RNG_WORDS * RNG_WORDS;
      uint32_t acc = 0;
      for ( int c = 0; c < RNG_WORDS; ++c )
      {
         const uint32_t sc = __shfl_sync(0xffffffffu, s, c);
         if ( lane < RNG_WORDS ) acc += M[c * RNG_WORDS + lane] * sc;
      }
      s = acc;
   }
   return s;
}

/* Jump the glibc state to output position `pos` and store it interleaved for lane `slot`. */
__device__ inline void warp_rng_jump(const DevData& D, uint64_t pos, uint32_t* ring, int slot, int lane)
{
   const uint32_t s = warp_rng_state(D, pos, lane);
   if ( lane < RNG_WORDS ) ring[lane * TILE + slot] = s;
}

/* ------------------------------------------------------ warp-coop steps */

/* fetchPair for pair (x, y) into column `j` of the tile's interleaved arrays
 * (STR = TILE), or into the pair's own contiguous arrays (STR = 1, j = 0). */
template <int STR = TILE>
__device__ inline int warp_fetch(const DevParams& P, const DevData& D, int32_t x, int32_t y, float2* X,
                          int8_t* lbl, int j, int lane)
{
   const float* g1 = D.gem + (size_t)x * P.S;
   const float* g2 = D.gem + (size_t)y * P.S;
   constexpr int CH = 4;            /* 32-sample chunks whose loads are in flight together */
   int n = 0;
   for ( int base = 0; base < P.S; base += CH * 32 )
   {
      float v1[CH], v2[CH];
#pragma unroll
      for ( int u = 0; u < CH; ++u )
      {
         const int s = base + u * 32 + lane;
         v1[u] = s < P.S ? __ldg(g1 + s) : 0.f;
         v2[u] = s < P.S ? __ldg(g2 + s) : 0.f;
      }
#pragma unroll
      for ( int u = 0; u < CH; ++u )
      {
         if ( base + u * 32 >= P.S ) break;   /* uniform over the warp */
         const int s = base + u * 32 + lane;
         bool use = false;
         if ( s < P.S )
         {
            const bool nanb = isnan(v1[u]) || isnan(v2[u]);
            const bool low = v1[u] < P.min_expr || v2[u] < P.min_expr;
            lbl[s * STR + j] = nanb ? (int8_t)-9 : (low ? (int8_t)-6 : (int8_t)0);
            use = !nanb && !low;
         }
         const unsigned bal = __ballot_sync(0xffffffffu, use);
         if ( use ) X[(n + __popc(bal & lanemask_lt())) * STR + j] = make_float2(v1[u], v2[u]);
         n += __popc(bal);
      }
   }
   __syncwarp();
   return n;
}

/* Clustering::markOutliers on column j of the tile (labels by sample position
 * i < N, values from the packed array at i, as in the reference); STR as in
 * warp_fetch. */
template <int STR = TILE>
__device__ inline void warp_mark_outliers(const float2* X, int N, int col, int8_t* lbl, int8_t cluster,
                                   int8_t marker, float* buf, int j, int lane)
{
   int n = 0;
   for ( int base = 0; base < N; base += 32 )
   {
      const int i = base + lane;
      bool sel = false;
      float v = 0.f;
      if ( i < N )
      {
         const int8_t l = lbl[i * STR + j];
         sel = l == cluster || l == marker;
         if ( sel )
         {
            const float2 xv = X[i * STR + j];
            v = col == 0 ? xv.x : xv.y;
         }
      }
      const unsigned bal = __ballot_sync(0xffffffffu, sel);
      if ( sel ) buf[n + __popc(bal & lanemask_lt())] = v;
      n += __popc(bal);
   }
   if ( n == 0 )
   {
      __syncwarp();
      return;
   }
   const int np2 = next_pow2(n);
   for ( int i = n + lane; i < np2; i += 32 ) buf[i] = __int_as_float(0x7f800000);
   __syncwarp();
   warp_bitonic(np2, buf, nullptr, lane);
   const float Q1 = buf[n * 1 / 4];
   const float Q3 = buf[n * 3 / 4];
   const float T_min = Q1 - 1.5f * (Q3 - Q1);
   const float T_max = Q3 + 1.5f * (Q3 - Q1);
   __syncwarp();
   for ( int i = lane; i < N; i += 32 )
   {
      if ( lbl[i * STR + j] == cluster )
      {
         const float2 xv = X[i * STR + j];
         const float v = col == 0 ? xv.x : xv.y;
         if ( v < T_min || T_max < v ) lbl[i * STR + j] = marker;
      }
   }
   __syncwarp();
}

/* Spearman::computeCluster for column j, cluster k; STR as in warp_fetch. */
template <int STR = TILE>
__device__ inline float warp_spearman(const DevParams& P, const DevData& D, const float2* X, const int8_t* lbl,
                               int32_t x, int32_t y, int8_t k, float* buf, int j, int lane)
{
   float* sx = buf;
   float* sy = buf + P.P2;
   float* sr = buf + 2 * P.P2;
   const float* g1 = D.gem + (size_t)x * P.S;
   const float* g2 = D.gem + (size_t)y * P.S;
   int n = 0;
   int jw = 0;
   for ( int base = 0; base < P.S; base += 32 )
   {
      const int i = base + lane;
      const int8_t l = i < P.S ? lbl[i * STR + j] : (int8_t)-1;
      const bool nonneg = l >= 0;
      const bool incl = l == k;
      const unsigned bn = __ballot_sync(0xffffffffu, nonneg);
      const unsigned bi = __ballot_sync(0xffffffffu, incl);
      if ( incl )
      {
         const int slot = n + __popc(bi & lanemask_lt());
         float2 v;
         if ( P.semantics == 0 )
         {
            v = X[(jw + __popc(bn & lanemask_lt())) * STR + j];
         }
         else
         {
            v = make_float2(g1[i], g2[i]);
         }
         sx[slot] = v.x;
         sy[slot] = v.y;
         sr[slot] = (float)(slot + 1);
      }
      n += __popc(bi);
      jw += __popc(bn);
   }
   if ( n < P.min_samples )
   {
      __syncwarp();
      return __int_as_float(0x7fc00000);
   }
   const int np2 = next_pow2(n);
   for ( int i = n + lane; i < np2; i += 32 )
   {
      sx[i] = __int_as_float(0x7f800000);
      sy[i] = __int_as_float(0x7f800000);
      sr[i] = 0.f;
   }
   __syncwarp();
   warp_bitonic(np2, sx, sy, lane);
   warp_bitonic(np2, sy, sr, lane);
   uint32_t diff = 0;
   for ( int i = lane; i < n; i += 32 )
   {
      const int tmp = (int)((float)(i + 1) - sr[i]);
      diff += (uint32_t)(tmp * tmp);
   }
   for ( int o = 16; o > 0; o >>= 1 ) diff += __shfl_xor_sync(0xffffffffu, diff, o);
   __syncwarp();
   const int32_t denom = (int32_t)((uint32_t)n * ((uint32_t)n * (uint32_t)n - 1u));
   return (float)(1.0 - 6.0 * (double)(int32_t)diff / (double)denom);
}

/* ------------------------------------------------------ lane-local fits */

/* A lane's per-component parameter array: registers, or (SMEM) a lane-strided
 * shared-memory column read at every use, which frees the registers for more
 * resident warps. */
template <int KA, bool SMEM> struct ParamArr;
template <int KA> struct ParamArr<KA, false>
{
   float v[KA];
   __device__ __forceinline__ ParamArr(float*, int) {}
   __device__ __forceinline__ float& operator[](int k) { return v[k]; }
};
template <int KA> struct ParamArr<KA, true>
{
   PARAM_QUAL float* p;
   __device__ __forceinline__ ParamArr(float* base, int which) : p(base + which * KA * TILE) {}
   __device__ __forceinline__ PARAM_QUAL float& operator[](int k) { return p[k * TILE]; }
};

__device__ __forceinline__ float log_mvn(float x0, float x1, float m0, float m1, float a, float b, float c,
                                         float nrm)
{
   /* calcLogMvNorm (pairwise_gmm.cpp:54-77) with the symmetric inverse [a b; b c] */
   const float xm0 = x0 - m0;
   const float xm1 = x1 - m1;
   const float b0 = a * xm0 + b * xm1;
   const float b1 = b * xm0 + c * xm1;
   const float dot = xm0 * b0 + xm1 * b1;
   return nrm - 0.5f * dot;
}

/* matrixInverse + prepareCovariance (pairwise_linalg.cpp:163-173, pairwise_gmm.cpp:31-47).  The
 * CPU code fails on det <= 0; the OpenCL kernel (OCL: GMM_Component_prepareCovariance,
 * src/opencl/gmm.cl:46-64) only on fabs(det) <= 0, and goes on with the NaN normaliser of a
 * negative determinant. */
template <bool OCL>
__device__ __forceinline__ bool prepare_cov(float s00, float s01, float s11, double c2, float& a, float& b,
                                            float& c, float& nrm)
{
   const float det = s00 * s11 - s01 * s01;
   a = s11 / det;
   b = -s01 / det;
   c = s00 / det;
   if ( OCL ? (fabsf(det) <= 0.f) : (det <= 0) ) return false;
   nrm = (float)(-0.5 * (c2 + (double)kinc_logf(det)));
   return true;
}

/*
 * GMM::fit for one pair on this lane (pairwise_gmm.cpp:367-445); with OCL, the OpenCL kernel's
 * GMM_fit (src/opencl/gmm.cl:424-495), which differs only in prepare_cov's failure rule.
 * Per EM iteration it makes three passes over the samples: E (log-densities,
 * per-sample log-sum-exp, logL, and the per-component maxima calcLogGammaK
 * needs), M1 (per-component log-sum-exp of the responsibilities, and the mean
 * sums) and M2 (covariance sums around the new means).  loggamma is not
 * stored: M1 recomputes it bit-identically from the parameters of the E step
 * (the inverse covariances and normalisers only change after M2, the new
 * means are held apart until then) and the stored per-sample log p(x); M1
 * keeps the responsibilities it forms for M2 (KINC_STORE_GAMMA).  Each
 * accumulator is still summed in sample order, so every value equals the
 * reference's.  The update of the last iteration is only checked (a
 * non-positive determinant still fails the fit), since the reference labels
 * samples with that iteration's E-step responsibilities.
 */
template <int KT, bool OCL>
__device__ bool gmm_fit(const float2* X, float* lpx, float* gam, int8_t* wl, int N, int Kr, LaneRng& rng,
                        double c2, float& out_logL, float& out_E, unsigned long long& units, float* pbuf, int pd)
{
   const int K = (KINC_STATIC_K && KT > 0) ? KT : Kr;
   /* KT > 0: up to KT components in registers (K <= KT at run time);
    * KT == 0: any K <= 64 from local memory.  M2 recomputes the
    * responsibilities of M1 unless KINC_STORE_GAMMA keeps them in
    * gam[(i*KT + k)*32] */
   constexpr int KA = KT > 0 ? KT : 64;
   constexpr int UF = KT > 0 ? KT : 1;
   constexpr bool STORE_G = KT > 0 && KINC_STORE_GAMMA;
   /* the E step's log(gamma/pi) in the same buffer: M1 reads it (no second log-density, no log p(x)),
    * overwrites it with gamma for M2; the label pass reads what is left, exactly the values the
    * reference's loggamma array holds when EM stops */
   constexpr bool STORE_V = STORE_G && KINC_STORE_LOGGAMMA;
   constexpr int SU = (KT > 0 && KT <= KINC_UNROLL_SMALL_K) ? 2 : SAMPLE_UNROLL;
   constexpr bool PS = KINC_GMM_PARAMS_SMEM && KT > 0;
   ParamArr<KA, PS> m0(pbuf, 0), m1(pbuf, 1), ia(pbuf, 2), ib(pbuf, 3), ic(pbuf, 4), nrm(pbuf, 5), logpi(pbuf, 6);

   if ( rng.mode == 1 ) rng.lcg = 1;
   {
      float a0, b0, c0, n0;
      prepare_cov<OCL>(1.f, 0.f, 1.f, c2, a0, b0, c0, n0);
      const float lp0 = kinc_logf(1.0f / K);
#pragma unroll UF
      for ( int k = 0; k < KA; ++k )
      {
         if ( k >= K ) continue;
         const int ii = rng.next() % N;
         const float2 xv = X[ii * TILE];
         m0[k] = xv.x;
         m1[k] = xv.y;
         ia[k] = a0; ib[k] = b0; ic[k] = c0; nrm[k] = n0;
         logpi[k] = lp0;
      }
   }

   float prevL = -INFINITY;
   float curL = -INFINITY;
   bool converged = false;
   for ( int t = 0; t < 100; ++t )
   {
      units += (unsigned long long)N * K;
      /* ---- E step */
      float logL = 0.0f;
      float maxG[KA];
#pragma unroll UF
      for ( int k = 0; k < KA; ++k )
      {
         if ( k >= K ) continue;
         maxG[k] = -INFINITY;
      }
      float2 xn = X[0];
      #pragma unroll SU
      for ( int i = 0; i < N; ++i )
      {
         const float2 xv = xn;
         if ( i + 1 < N ) xn = X[(i + 1) * TILE];
         if ( pd > 0 && i + pd < N ) prefetch_l2(&X[(i + pd) * TILE]);
         float lg[KA];
         float m = -INFINITY;
#pragma unroll UF
         for ( int k = 0; k < KA; ++k )
         {
            if ( k >= K ) continue;
            lg[k] = log_mvn(xv.x, xv.y, m0[k], m1[k], ia[k], ib[k], ic[k], nrm[k]);
            const float lp = logpi[k] + lg[k];
            if ( lp > m ) m = lp;
         }
         float sum = 0.0f;
#pragma unroll UF
         for ( int k = 0; k < KA; ++k )
         {
            if ( k >= K ) continue;
            sum += kinc_expf((logpi[k] + lg[k]) - m);
         }
         const float logpx = m + kinc_logf(sum);
         logL += logpx;
         if ( !STORE_V ) lpx[i * TILE] = logpx;
#pragma unroll UF
         for ( int k = 0; k < KA; ++k )
         {
            if ( k >= K ) continue;
            const float v = lg[k] + (-logpx);
            if ( v > maxG[k] ) maxG[k] = v;
            if ( STORE_V ) gam[(i * KA + k) * TILE] = v;
         }
      }
      prevL = curL;
      curL = logL;
      if ( fabsf(curL - prevL) < 1e-8f )
      {
         converged = true;
         break;
      }

      /* ---- M step, pass 1: logGamma sums and mean sums */
      float nm0[KA], nm1[KA], Gam[KA];
      {
         float sG[KA];
#pragma unroll UF
         for ( int k = 0; k < KA; ++k )
         {
            if ( k >= K ) continue;
            sG[k] = 0.f; nm0[k] = 0.f; nm1[k] = 0.f;
         }
         xn = X[0];
         float ln = STORE_V ? 0.f : lpx[0];
         #pragma unroll SU
         for ( int i = 0; i < N; ++i )
         {
            const float2 xv = xn;
            const float logpx = ln;
            if ( i + 1 < N )
            {
               xn = X[(i + 1) * TILE];
               if ( !STORE_V ) ln = lpx[(i + 1) * TILE];
            }
            if ( pd > 0 && i + pd < N )
            {
               prefetch_l2(&X[(i + pd) * TILE]);
               if ( STORE_V )
               {
#pragma unroll UF
                  for ( int k = 0; k < KA; ++k )
                  {
                     if ( k >= K ) continue;
                     prefetch_l2(&gam[((i + pd) * KA + k) * TILE]);
                  }
               }
               else
               {
                  prefetch_l2(&lpx[(i + pd) * TILE]);
               }
            }
#pragma unroll UF
            for ( int k = 0; k < KA; ++k )
            {
               if ( k >= K ) continue;
               const float lgk = STORE_V ? gam[(i * KA + k) * TILE]
                                         : log_mvn(xv.x, xv.y, m0[k], m1[k], ia[k], ib[k], ic[k], nrm[k]) + (-logpx);
               sG[k] += kinc_expf(lgk - maxG[k]);
               const float g = kinc_expf(lgk);
               if ( STORE_G ) gam[(i * KA + k) * TILE] = g;
               nm0[k] += g * xv.x;
               nm1[k] += g * xv.y;
            }
         }
         float logGamma[KA];
         float mx = -INFINITY;
#pragma unroll UF
         for ( int k = 0; k < KA; ++k )
         {
            if ( k >= K ) continue;
            logGamma[k] = maxG[k] + kinc_logf(sG[k]);
            const float arg = logpi[k] + logGamma[k];
            if ( arg > mx ) mx = arg;
         }
         float s = 0.f;
#pragma unroll UF
         for ( int k = 0; k < KA; ++k )
         {
            if ( k >= K ) continue;
            s += kinc_expf((logpi[k] + logGamma[k]) - mx);
         }
         const float lgs = mx + kinc_logf(s);
#pragma unroll UF
         for ( int k = 0; k < KA; ++k )
         {
            if ( k >= K ) continue;
            logpi[k] += logGamma[k] - lgs;
            Gam[k] = kinc_expf(logGamma[k]);
            const float sc = 1.0f / Gam[k];
            nm0[k] = nm0[k] * sc;
            nm1[k] = nm1[k] * sc;
         }
      }

      /* ---- M step, pass 2: covariance sums around the new means */
      float s00[KA], s01[KA], s11[KA];
#pragma unroll UF
      for ( int k = 0; k < KA; ++k )
      {
         if ( k >= K ) continue;
         s00[k] = 0.f; s01[k] = 0.f; s11[k] = 0.f;
      }
      xn = X[0];
      float ln = lpx[0];
      /* kept responsibilities of sample i+1 loaded while sample i is summed (static K only) */
      constexpr bool PIPE_G = STORE_G && KT > 0 && KINC_GMM_PIPE_G;
      float gn[PIPE_G ? KA : 1];
      if ( PIPE_G )
      {
#pragma unroll UF
         for ( int k = 0; k < KA; ++k )
         {
            if ( k >= K ) continue;
            gn[k] = gam[k * TILE];
         }
      }
      #pragma unroll SU
      for ( int i = 0; i < N; ++i )
      {
         const float2 xv = xn;
         const float logpx = ln;
         float gc[PIPE_G ? KA : 1];
         if ( PIPE_G )
         {
#pragma unroll UF
            for ( int k = 0; k < KA; ++k )
            {
               if ( k >= K ) continue;
               gc[k] = gn[k];
            }
         }
         if ( i + 1 < N )
         {
            xn = X[(i + 1) * TILE];
            ln = lpx[(i + 1) * TILE];
            if ( PIPE_G )
            {
#pragma unroll UF
               for ( int k = 0; k < KA; ++k )
               {
                  if ( k >= K ) continue;
                  gn[k] = gam[((i + 1) * KA + k) * TILE];
               }
            }
         }
         if ( pd > 0 && i + pd < N )
         {
            prefetch_l2(&X[(i + pd) * TILE]);
            if ( STORE_G )
            {
#pragma unroll UF
               for ( int k = 0; k < KA; ++k )
               {
                  if ( k >= K ) continue;
                  prefetch_l2(&gam[((i + pd) * KA + k) * TILE]);
               }
            }
            else
            {
               prefetch_l2(&lpx[(i + pd) * TILE]);
            }
         }
#pragma unroll UF
         for ( int k = 0; k < KA; ++k )
         {
            if ( k >= K ) continue;
            float g;
            if ( PIPE_G )
            {
               g = gc[k];
            }
            else if ( STORE_G )
            {
               g = gam[(i * KA + k) * TILE];
            }
            else
            {
               const float lgk = log_mvn(xv.x, xv.y, m0[k], m1[k], ia[k], ib[k], ic[k], nrm[k]) + (-logpx);
               g = kinc_expf(lgk);
            }
            const float xm0 = xv.x - nm0[k];
            const float xm1 = xv.y - nm1[k];
            s00[k] += g * (xm0 * xm0);
            s01[k] += g * (xm0 * xm1);
            s11[k] += g * (xm1 * xm1);
         }
      }
      bool ok = true;
      const bool last = t == 99;
#pragma unroll UF
      for ( int k = 0; k < KA; ++k )
      {
         if ( k >= K ) continue;
         const float sc = 1.0f / Gam[k];
         float a, b, c, n;
         ok = prepare_cov<OCL>(s00[k] * sc, s01[k] * sc, s11[k] * sc, c2, a, b, c, n) && ok;
         if ( !last )
         {
            m0[k] = nm0[k]; m1[k] = nm1[k];
            ia[k] = a; ib[k] = b; ic[k] = c; nrm[k] = n;
         }
      }
      if ( !ok ) return false;
   }

   /* ---- calcLabels + calcEntropy on what the reference's loggamma array holds:
    * log(gamma/pi) of the last E step if EM converged, exp of it if it ran out
    * of iterations (the parameters still are that E step's in both cases) */
   out_logL = curL;
   float E = 0.f;
   for ( int i = 0; i < N; ++i )
   {
      const float2 xv = STORE_V ? make_float2(0.f, 0.f) : X[i * TILE];
      const float logpx = STORE_V ? 0.f : lpx[i * TILE];
      int max_k = -1;
      float max_g = -INFINITY;
#pragma unroll UF
      for ( int k = 0; k < KA; ++k )
      {
         if ( k >= K ) continue;
         float v;
         if ( STORE_V )
         {
            v = gam[(i * KA + k) * TILE];   /* log(gamma/pi) if converged, else the last M1's exp of it */
         }
         else
         {
            v = log_mvn(xv.x, xv.y, m0[k], m1[k], ia[k], ib[k], ic[k], nrm[k]) + (-logpx);
            if ( !converged ) v = kinc_expf(v);
         }
         if ( max_g < v )
         {
            max_k = k;
            max_g = v;
         }
      }
      wl[i * TILE] = (int8_t)max_k;
      E += max_k >= 0 ? kinc_logf(max_g) : __int_as_float(0x7fc00000);
   }
   out_E = E;
   return true;
}

/* calcLogMvNorm for one component (float) or two (F2), the operations of log_mvn; every product
 * that feeds a sum goes through mulz, so it is rounded on its own as in the reference */
template <class T>
__device__ __forceinline__ T log_mvn_t(T x0, T x1, T m0, T m1, T a, T b, T c, T nrm, T z)
{
   const T xm0 = x0 - m0;
   const T xm1 = x1 - m1;
   const T b0 = mulz(a, xm0, z) + mulz(b, xm1, z);
   const T b1 = mulz(b, xm0, z) + mulz(c, xm1, z);
   const T dot = mulz(xm0, b0, z) + mulz(xm1, b1, z);
   return nrm - mulz(cst<T>(0.5f), dot, z);
}

/* K per-component floats held as K/2 packed pairs (components 2q, 2q+1) and, for odd K, one
 * float (component K-1); element access with a compile-time k reads or writes half a register */
template <int K>
struct PArr
{
   static constexpr int NP = K / 2;
   F2 p[NP > 0 ? NP : 1];
   float o;
   __device__ __forceinline__ float get(int k) const
   {
      if ( k == K - 1 && (K & 1) ) return o;
      return (k & 1) ? hi(p[k >> 1]) : lo(p[k >> 1]);
   }
   __device__ __forceinline__ void set(int k, float v)
   {
      if ( k == K - 1 && (K & 1) )
         o = v;
      else if ( k & 1 )
         p[k >> 1] = f2(lo(p[k >> 1]), v);
      else
         p[k >> 1] = f2(v, hi(p[k >> 1]));
   }
   __device__ __forceinline__ void fill(float v)
   {
#pragma unroll
      for ( int q = 0; q < NP; ++q ) p[q] = f2(v);
      o = v;
   }
};

/*
 * gmm_fit with the mixture components paired in packed FP32 registers: components (2q, 2q+1)
 * share one F2 for every per-component value of the three EM passes, and an odd last component
 * runs in plain floats.  Every per-component operation is the one gmm_fit performs, on each half,
 * every accumulator is still summed in sample order, and the cross-component steps (maximum,
 * the log-sum-exp sum in component order, the E-step's log) stay scalar, so the results are
 * gmm_fit's bit for bit with about half the floating-point instructions issued.
 * Responsibilities are kept between M1 and M2 as gmm_fit keeps them, laid out per sample as
 * [pair q][lane][2] followed by the odd component's [lane] (KT x 32 floats per sample as before).
 */
template <int KT, bool OCL>
__device__ bool gmm_fit_packed(const float2* X, float* lpx, float* gam, int8_t* wl, int N, LaneRng& rng, double c2,
                               float& out_logL, float& out_E, unsigned long long& units, int pd, float neg_zero)
{
   static_assert(KT >= 2, "one component has nothing to pair");
   constexpr int K = KT;
   constexpr int NP = KT / 2;
   constexpr bool ODD = (KT & 1) != 0;
   constexpr int GS = KT * TILE;               /* floats of gam per sample */
   const int lane = threadIdx.x & 31;
   /* gam = slot base + lane: pair q of sample i at base + i*GS + q*64 + 2*lane, the odd
    * component at base + i*GS + NP*64 + lane */
   float* gpair = gam + lane;
   float* godd = gam + NP * 2 * TILE;
   const F2 z = f2(neg_zero);
   constexpr int GR = KINC_GMM_RING;           /* samples the E and M1 sweeps keep in flight */
   constexpr int EU = KINC_GMM_E_UNROLL;
   constexpr int M2U = KINC_GMM_M2_UNROLL;

   PArr<K> m0, m1, ia, ib, ic, nrm, logpi;
   if ( rng.mode == 1 ) rng.lcg = 1;
   {
      float a0, b0, c0, n0;
      prepare_cov<OCL>(1.f, 0.f, 1.f, c2, a0, b0, c0, n0);
      ia.fill(a0); ib.fill(b0); ic.fill(c0); nrm.fill(n0);
      logpi.fill(kinc_logf(1.0f / K));
#pragma unroll
      for ( int k = 0; k < K; ++k )
      {
         const int ii = rng.next() % N;
         const float2 xv = X[ii * TILE];
         m0.set(k, xv.x);
         m1.set(k, xv.y);
      }
   }

   float prevL = -INFINITY;
   float curL = -INFINITY;
   bool converged = false;
   for ( int t = 0; t < 100; ++t )
   {
      units += (unsigned long long)N * K;

      /* ---- E step */
      float logL = 0.0f;
      PArr<K> maxG;
      maxG.fill(-INFINITY);
      /* the next GR samples in flight in registers */
      float2 xr[GR];
#pragma unroll
      for ( int d = 0; d < GR; ++d ) xr[d] = d < N ? X[d * TILE] : make_float2(0.f, 0.f);
#pragma unroll EU
      for ( int i = 0; i < N; ++i )
      {
         const float2 xv = xr[0];
#pragma unroll
         for ( int d = 0; d + 1 < GR; ++d ) xr[d] = xr[d + 1];
         if ( i + GR < N ) xr[GR - 1] = X[(i + GR) * TILE];
         if ( pd > 0 && i + pd < N ) prefetch_l2(&X[(i + pd) * TILE]);
         const F2 x0 = f2(xv.x), x1 = f2(xv.y);
         F2 lg[NP], lp[NP];
         float lgo = 0.f, lpo = 0.f;
         float m = -INFINITY;
#pragma unroll
         for ( int q = 0; q < NP; ++q )
         {
            lg[q] = log_mvn_t(x0, x1, m0.p[q], m1.p[q], ia.p[q], ib.p[q], ic.p[q], nrm.p[q], z);
            lp[q] = logpi.p[q] + lg[q];
            float a, b;
            split(lp[q], a, b);
            /* fmaxf keeps m where a comparison would (m is never NaN; m's zero sign changes no result) */
            m = fmaxf(m, a);
            m = fmaxf(m, b);
         }
         if ( ODD )
         {
            lgo = log_mvn(xv.x, xv.y, m0.o, m1.o, ia.o, ib.o, ic.o, nrm.o);
            lpo = logpi.o + lgo;
            m = fmaxf(m, lpo);
         }
         float sum = 0.0f;
         const F2 mm = f2(m);
#pragma unroll
         for ( int q = 0; q < NP; ++q )
         {
            float a, b;
            split(kinc_expf2(lp[q] - mm), a, b);
            sum += a;
            sum += b;
         }
         if ( ODD ) sum += kinc_expf(lpo - m);
         const float logpx = m + kinc_logf(sum);
         logL += logpx;
         lpx[i * TILE] = logpx;
         const F2 nl = f2(-logpx);
#pragma unroll
         for ( int q = 0; q < NP; ++q )
         {
            float a, b, ga, gb;
            split(lg[q] + nl, a, b);
            split(maxG.p[q], ga, gb);
            maxG.p[q] = f2(fmaxf(ga, a), fmaxf(gb, b));
         }
         if ( ODD )
         {
            maxG.o = fmaxf(maxG.o, lgo + (-logpx));
         }
      }
      prevL = curL;
      curL = logL;
      if ( fabsf(curL - prevL) < 1e-8f )
      {
         converged = true;
         break;
      }

      /* ---- M step, pass 1: logGamma sums and mean sums */
      PArr<K> nm0, nm1, Gam;
      {
         PArr<K> sG;
         sG.fill(0.f);
         nm0.fill(0.f);
         nm1.fill(0.f);
         float2 xr[GR];
         float lr[GR];
#pragma unroll
         for ( int d = 0; d < GR; ++d )
         {
            xr[d] = d < N ? X[d * TILE] : make_float2(0.f, 0.f);
            lr[d] = d < N ? lpx[d * TILE] : 0.f;
         }
         for ( int i = 0; i < N; ++i )
         {
            const float2 xv = xr[0];
            const float logpx = lr[0];
#pragma unroll
            for ( int d = 0; d + 1 < GR; ++d )
            {
               xr[d] = xr[d + 1];
               lr[d] = lr[d + 1];
            }
            if ( i + GR < N )
            {
               xr[GR - 1] = X[(i + GR) * TILE];
               lr[GR - 1] = lpx[(i + GR) * TILE];
            }
            if ( pd > 0 && i + pd < N )
            {
               prefetch_l2(&X[(i + pd) * TILE]);
               prefetch_l2(&lpx[(i + pd) * TILE]);
            }
            const F2 x0 = f2(xv.x), x1 = f2(xv.y), nl = f2(-logpx);
#pragma unroll
            for ( int q = 0; q < NP; ++q )
            {
               const F2 lgk = log_mvn_t(x0, x1, m0.p[q], m1.p[q], ia.p[q], ib.p[q], ic.p[q], nrm.p[q], z) + nl;
               sG.p[q] += kinc_expf2(lgk - maxG.p[q]);
               const F2 g = kinc_expf2(lgk);
               *reinterpret_cast<unsigned long long*>(gpair + i * GS + q * 2 * TILE) = g.v;
               nm0.p[q] += mulz(g, x0, z);
               nm1.p[q] += mulz(g, x1, z);
            }
            if ( ODD )
            {
               const float lgk = log_mvn(xv.x, xv.y, m0.o, m1.o, ia.o, ib.o, ic.o, nrm.o) + (-logpx);
               sG.o += kinc_expf(lgk - maxG.o);
               const float g = kinc_expf(lgk);
               godd[i * GS] = g;
               nm0.o += g * xv.x;
               nm1.o += g * xv.y;
            }
         }
         float logGamma[K];
         float mx = -INFINITY;
#pragma unroll
         for ( int k = 0; k < K; ++k )
         {
            logGamma[k] = maxG.get(k) + kinc_logf(sG.get(k));
            const float arg = logpi.get(k) + logGamma[k];
            if ( arg > mx ) mx = arg;
         }
         float s = 0.f;
#pragma unroll
         for ( int k = 0; k < K; ++k ) s += kinc_expf((logpi.get(k) + logGamma[k]) - mx);
         const float lgs = mx + kinc_logf(s);
#pragma unroll
         for ( int k = 0; k < K; ++k )
         {
            logpi.set(k, logpi.get(k) + (logGamma[k] - lgs));
            const float G = kinc_expf(logGamma[k]);
            Gam.set(k, G);
            const float sc = 1.0f / G;
            nm0.set(k, nm0.get(k) * sc);
            nm1.set(k, nm1.get(k) * sc);
         }
      }

      /* ---- M step, pass 2: covariance sums around the new means */
      PArr<K> s00, s01, s11;
      s00.fill(0.f);
      s01.fill(0.f);
      s11.fill(0.f);
      /* the pass does little arithmetic per sample, so sample i+1's point and responsibilities are
       * loaded while sample i is summed */
      float2 xn = X[0];
      F2 gn[NP];
      float gno = 0.f;
#pragma unroll
      for ( int q = 0; q < NP; ++q ) gn[q].v = *reinterpret_cast<const unsigned long long*>(gpair + q * 2 * TILE);
      if ( ODD ) gno = godd[0];
#pragma unroll M2U
      for ( int i = 0; i < N; ++i )
      {
         const float2 xv = xn;
         F2 gc[NP];
#pragma unroll
         for ( int q = 0; q < NP; ++q ) gc[q] = gn[q];
         const float gco = gno;
         if ( i + 1 < N )
         {
            xn = X[(i + 1) * TILE];
#pragma unroll
            for ( int q = 0; q < NP; ++q )
               gn[q].v = *reinterpret_cast<const unsigned long long*>(gpair + (i + 1) * GS + q * 2 * TILE);
            if ( ODD ) gno = godd[(i + 1) * GS];
         }
         if ( pd > 0 && i + pd < N )
         {
            prefetch_l2(&X[(i + pd) * TILE]);
#pragma unroll
            for ( int q = 0; q < NP; ++q ) prefetch_l2(gpair + (i + pd) * GS + q * 2 * TILE);
            if ( ODD ) prefetch_l2(godd + (i + pd) * GS);
         }
         const F2 x0 = f2(xv.x), x1 = f2(xv.y);
#pragma unroll
         for ( int q = 0; q < NP; ++q )
         {
            const F2 g = gc[q];
            const F2 xm0 = x0 - nm0.p[q];
            const F2 xm1 = x1 - nm1.p[q];
            s00.p[q] += mulz(g, xm0 * xm0, z);
            s01.p[q] += mulz(g, xm0 * xm1, z);
            s11.p[q] += mulz(g, xm1 * xm1, z);
         }
         if ( ODD )
         {
            const float g = gco;
            const float xm0 = xv.x - nm0.o;
            const float xm1 = xv.y - nm1.o;
            s00.o += g * (xm0 * xm0);
            s01.o += g * (xm0 * xm1);
            s11.o += g * (xm1 * xm1);
         }
      }
      bool ok = true;
      const bool last = t == 99;
#pragma unroll
      for ( int k = 0; k < K; ++k )
      {
         const float sc = 1.0f / Gam.get(k);
         float a, b, c, n;
         ok = prepare_cov<OCL>(s00.get(k) * sc, s01.get(k) * sc, s11.get(k) * sc, c2, a, b, c, n) && ok;
         if ( !last )
         {
            m0.set(k, nm0.get(k));
            m1.set(k, nm1.get(k));
            ia.set(k, a); ib.set(k, b); ic.set(k, c); nrm.set(k, n);
         }
      }
      if ( !ok ) return false;
   }

   /* ---- calcLabels + calcEntropy, as gmm_fit */
   out_logL = curL;
   float E = 0.f;
   for ( int i = 0; i < N; ++i )
   {
      const float2 xv = X[i * TILE];
      const float logpx = lpx[i * TILE];
      int max_k = -1;
      float max_g = -INFINITY;
#pragma unroll
      for ( int k = 0; k < K; ++k )
      {
         float v = log_mvn(xv.x, xv.y, m0.get(k), m1.get(k), ia.get(k), ib.get(k), ic.get(k), nrm.get(k)) +
                   (-logpx);
         if ( !converged ) v = kinc_expf(v);
         if ( max_g < v )
         {
            max_k = k;
            max_g = v;
         }
      }
      wl[i * TILE] = (int8_t)max_k;
      E += max_k >= 0 ? kinc_logf(max_g) : __int_as_float(0x7fc00000);
   }
   out_E = E;
   return true;
}

/* "no label changed": a lane's label columns ya and yb (stride TILE) agree on samples [0, N).
 * The whole range is compared without an early exit, so the loads of several samples are in flight
 * at once (the first mismatch decides nothing that the full comparison does not). */
__device__ __forceinline__ bool labels_equal(const int8_t* ya, const int8_t* yb, int N)
{
   bool same = true;
#pragma unroll 8
   for ( int i = 0; i < N; ++i ) same &= ya[i * TILE] == yb[i * TILE];
   return same;
}

/* vectorDiffNorm (pairwise_linalg.cpp:97-104) */
__device__ __forceinline__ float diff_norm(float x0, float x1, float m0, float m1)
{
   float dist = 0;
   dist += (x0 - m0) * (x0 - m0);
   dist += (x1 - m1) * (x1 - m1);
   return sqrtf(dist);
}

/* KMeans::fit for one pair on this lane (pairwise_kmeans.cpp:12-99).  The
 * best run's labels end up in *best (a pointer into the three buffers).
 * Each Lloyd iteration is one pass: the reference's mean update of an
 * iteration sums the samples under exactly the labels that iteration's
 * assignment produced, in sample order, so those sums are accumulated during
 * the assignment (and dropped when the labels did not change).  The first
 * iteration compares against the all-zero initial labels without reading them. */
template <int KT>
__device__ float kmeans_fit_inits_in_step(const float2* X, int8_t*& cur, int8_t*& nxt, int8_t*& best, int N, int Kr,
                            LaneRng& rng, unsigned long long& units)
{
   /* KT > 0: up to KT centroids in registers (K <= KT at run time);
    * KT == 0: any K <= 64 from local memory */
   const int K = (KINC_STATIC_K && KT > 0) ? KT : Kr;
   constexpr int KA = KT > 0 ? KT : 64;
   constexpr int UF = KT > 0 ? KT : 1;
   float bestLogL = -INFINITY;
   if ( rng.mode == 1 ) rng.lcg = 1;
   for ( int init = 0; init < 10; ++init )
   {
      float mu0[KA], mu1[KA];
#pragma unroll UF
      for ( int k = 0; k < KA; ++k )
      {
         if ( k >= K ) continue;
         const int ii = rng.next() % N;
         const float2 xv = X[ii * TILE];
         mu0[k] = xv.x;
         mu1[k] = xv.y;
      }
      int8_t* ya = cur;     /* labels of the previous iteration */
      int8_t* yb = nxt;     /* labels being assigned */
      bool first = true;    /* ya is the all-zero initial vector, not yet written */
      bool converged = false;
      int nprev[KA];        /* cluster sizes behind the current means */
#pragma unroll UF
      for ( int k = 0; k < KA; ++k ) nprev[k] = -1;
      for ( int t = 0; t < 300; ++t )
      {
         units += (unsigned long long)N * K;
         bool same = true;
         float s0[KA], s1[KA];
         int nk[KA];
#pragma unroll UF
         for ( int k = 0; k < KA; ++k )
         {
            if ( k >= K ) continue;
            s0[k] = 0.f; s1[k] = 0.f; nk[k] = 0;
         }
         /* the next KM_RING samples are in flight in registers (N >= min_samples >= 1) */
         float2 ring[KM_RING];
#pragma unroll
         for ( int d = 0; d < KM_RING; ++d ) ring[d] = d < N ? X[d * TILE] : make_float2(0.f, 0.f);
         for ( int i = 0; i < N; ++i )
         {
            const float2 xv = ring[0];
#pragma unroll
            for ( int d = 0; d + 1 < KM_RING; ++d ) ring[d] = ring[d + 1];
            if ( i + KM_RING < N ) ring[KM_RING - 1] = X[(i + KM_RING) * TILE];
            if ( KINC_PREFETCH > 0 && i + KINC_PREFETCH < N ) prefetch_l2(&X[(i + KINC_PREFETCH) * TILE]);
            int min_k = -1;
            float min_d = 0.f;
#pragma unroll UF
            for ( int k = 0; k < KA; ++k )
            {
               if ( k >= K ) continue;
               const float d = diff_norm(xv.x, xv.y, mu0[k], mu1[k]);
               if ( min_k == -1 || d < min_d )
               {
                  min_k = k;
                  min_d = d;
               }
            }
            yb[i * TILE] = (int8_t)min_k;
#pragma unroll UF
            for ( int k = 0; k < KA; ++k )
            {
               if ( k >= K ) continue;
               if ( k == min_k )
               {
                  s0[k] += xv.x;
                  s1[k] += xv.y;
                  nk[k]++;
               }
            }
         }
         /*
          * "no label changed", decided without reading the previous labels in the sweep:
          * first iteration: the previous labels are all zero, so unchanged <=> every sample in
          * cluster 0.  Later: the means are formed from the labels by the same ordered sums, so
          * unchanged labels give bit-identical means and counts; when those match, the label
          * arrays are compared to decide exactly.
          */
         float n0[KA], n1[KA];
         bool means_same = true;
#pragma unroll UF
         for ( int k = 0; k < KA; ++k )
         {
            if ( k >= K ) continue;
            const float sc = 1.0f / nk[k];
            n0[k] = s0[k] * sc;
            n1[k] = s1[k] * sc;
            means_same = means_same && __float_as_uint(n0[k]) == __float_as_uint(mu0[k])
                         && __float_as_uint(n1[k]) == __float_as_uint(mu1[k]) && nk[k] == nprev[k];
         }
         if ( first )
         {
            same = nk[0] == N;
         }
         else if ( means_same )
         {
            same = labels_equal(ya, yb, N);
         }
         else
         {
            same = false;
         }
         if ( same )
         {
            converged = true;
            break;
         }
         int8_t* tmp = ya;
         ya = yb;
         yb = tmp;
         first = false;
#pragma unroll UF
         for ( int k = 0; k < KA; ++k )
         {
            if ( k >= K ) continue;
            mu0[k] = n0[k];
            mu1[k] = n1[k];
            nprev[k] = nk[k];
         }
      }
      /* the labels: the unchanged assignment (in yb) if converged, else the last one (ya) */
      int8_t* lab = converged ? yb : ya;
      /* computeLogLikelihood: one accumulator, cluster-major order */
      float S = 0.f;
      for ( int k = 0; k < K; ++k )
      {
         float c0 = 0.f, c1 = 0.f;
#pragma unroll UF
         for ( int kk = 0; kk < KA; ++kk )
         {
            if ( kk >= K ) continue;
            if ( kk == k ) { c0 = mu0[kk]; c1 = mu1[kk]; }
         }
         for ( int i = 0; i < N; ++i )
         {
            if ( lab[i * TILE] != k ) continue;
            const float2 xv = X[i * TILE];
            const float d = diff_norm(xv.x, xv.y, c0, c1);
            S += d * d;
         }
      }
      const float logL = -S;
      /* keep the buffers distinct: cur/nxt are this run's, best the kept one */
      if ( bestLogL < logL )
      {
         bestLogL = logL;
         int8_t* old = best;
         best = lab;
         cur = (lab == cur) ? old : cur;
         nxt = (lab == nxt) ? old : nxt;
      }
   }
   return bestLogL;
}

/* 1: lane-independent initialisations (below); measured slower on the uneven 10,000 x 4,000 workload
 * (12.8k vs 15.0k pairs/s): the cluster-major log-likelihood pass of a lane that finishes an
 * initialisation then runs divergently beside the other lanes' Lloyd sweeps */
/* K-means sweeps over a per-lane contiguous copy of the samples (1) or the interleaved X (0).
 * (The label buffers stay interleaved: per-lane contiguous labels made every one-byte store of a
 * sweep touch its own line and measured 63.0k against 82.8k pairs/s.) */
#ifndef KINC_KMEANS_LANE_MAJOR
#define KINC_KMEANS_LANE_MAJOR 1
#endif

/* K-means initialisations pipelined across the lanes of a warp (below); 0: in lockstep */
#ifndef KINC_KMEANS_PIPELINE
#define KINC_KMEANS_PIPELINE 1
#endif

/* computeLogLikelihood (pairwise_kmeans.cpp:105-127): one accumulator, cluster-major order */
template <int KT, int XS = TILE>
__device__ __forceinline__ float kmeans_loglik(const float2* X, const int8_t* lab, int N, int K, const float* mu0,
                                               const float* mu1)
{
   constexpr int KA = KT > 0 ? KT : 64;
   constexpr int UF = KT > 0 ? KT : 1;
   float S = 0.f;
   for ( int k = 0; k < K; ++k )
   {
      float c0 = 0.f, c1 = 0.f;
#pragma unroll UF
      for ( int kk = 0; kk < KA; ++kk )
      {
         if ( kk >= K ) continue;
         if ( kk == k ) { c0 = mu0[kk]; c1 = mu1[kk]; }
      }
      for ( int i = 0; i < N; ++i )
      {
         if ( lab[i * TILE] != k ) continue;
         const float2 xv = X[i * XS];
         const float d = diff_norm(xv.x, xv.y, c0, c1);
         S += d * d;
      }
   }
   return -S;
}

/*
 * KMeans::fit (pairwise_kmeans.cpp:12-99) with the 10 initialisations of the
 * warp's lanes pipelined one deep.  A lane whose initialisation has converged
 * parks its result (labels and means) as "pending" and starts its next
 * initialisation at once, while slower lanes still iterate; the pending
 * results' log-likelihoods are computed together, by every lane at the same
 * time, when each lane holds one (or has nothing left to run).  A lane that
 * finishes a second initialisation before that waits.  Every lane draws its
 * means, iterates and compares log-likelihoods in exactly the reference's
 * order, so its results are those of the lockstep form; only the schedule
 * changes.  Four label buffers per lane: the running initialisation's two,
 * the pending one and the best so far (returned in `best`).
 *
 * Warp votes use the lanes that entered together (__activemask at entry);
 * every one of them runs the loop until the same voted exit.
 */
template <int KT, int XS = TILE>
__device__ float kmeans_fit_pipelined(const float2* X, int8_t*& ya, int8_t*& yb, int8_t*& pl, int8_t*& best,
                                      int N, int Kr, LaneRng& rng, unsigned long long& units)
{
   const int K = (KINC_STATIC_K && KT > 0) ? KT : Kr;
   constexpr int KA = KT > 0 ? KT : 64;
   constexpr int UF = KT > 0 ? KT : 1;
   const unsigned mask = __activemask();
   float bestLogL = -INFINITY;
   if ( rng.mode == 1 ) rng.lcg = 1;
   float mu0[KA], mu1[KA];      /* the running (or held) initialisation's means */
   float pm0[KA], pm1[KA];      /* the pending initialisation's means */
   int nprev[KA];
   int started = 0;             /* initialisations begun */
   bool running = false;        /* an initialisation is iterating */
   bool held = false;           /* a finished initialisation waits for the pending one */
   bool pending = false;
   bool first = true;
   int t = 0;
   int8_t* hl = nullptr;        /* labels of the held initialisation (ya or yb) */

   for ( ;; )
   {
      /* start the next initialisation where possible */
      if ( !running && !held && started < 10 )
      {
#pragma unroll UF
         for ( int k = 0; k < KA; ++k )
         {
            if ( k >= K ) continue;
            const int ii = rng.next() % N;
            const float2 xv = X[ii * XS];
            mu0[k] = xv.x;
            mu1[k] = xv.y;
            nprev[k] = -1;
         }
         ++started;
         running = true;
         first = true;
         t = 0;
      }
      const bool any_running = __any_sync(mask, running);
      const bool all_ready = __all_sync(mask, pending || (!running && !held && started >= 10));
      if ( !any_running || all_ready )
      {
         /* the pending results, all lanes together, in each lane's initialisation order */
         if ( __all_sync(mask, !pending && !held && !running && started >= 10) ) break;
         if ( pending )
         {
            const float logL = kmeans_loglik<KT, XS>(X, pl, N, K, pm0, pm1);
            if ( bestLogL < logL )
            {
               bestLogL = logL;
               int8_t* tmp = best;
               best = pl;
               pl = tmp;
            }
            pending = false;
         }
         if ( held )
         {
            /* the held result becomes the pending one; its buffer trades places with the free pending one */
            int8_t* tmp = pl;
            pl = hl;
            if ( hl == ya ) ya = tmp; else yb = tmp;
#pragma unroll UF
            for ( int k = 0; k < KA; ++k )
            {
               if ( k >= K ) continue;
               pm0[k] = mu0[k];
               pm1[k] = mu1[k];
            }
            pending = true;
            held = false;
         }
         continue;
      }
      if ( !running ) continue;

      /* one Lloyd iteration of the running initialisation (as in kmeans_fit_inits_in_step) */
      units += (unsigned long long)N * K;
      float s0[KA], s1[KA];
      int nk[KA];
#pragma unroll UF
      for ( int k = 0; k < KA; ++k )
      {
         if ( k >= K ) continue;
         s0[k] = 0.f; s1[k] = 0.f; nk[k] = 0;
      }
      float2 ring[KM_RING];
#pragma unroll
      for ( int d = 0; d < KM_RING; ++d ) ring[d] = d < N ? X[d * XS] : make_float2(0.f, 0.f);
      for ( int i = 0; i < N; ++i )
      {
         const float2 xv = ring[0];
#pragma unroll
         for ( int d = 0; d + 1 < KM_RING; ++d ) ring[d] = ring[d + 1];
         if ( i + KM_RING < N ) ring[KM_RING - 1] = X[(i + KM_RING) * XS];
         if ( XS != 1 && KINC_PREFETCH > 0 && i + KINC_PREFETCH < N ) prefetch_l2(&X[(i + KINC_PREFETCH) * XS]);
         int min_k = -1;
         float min_d = 0.f;
#pragma unroll UF
         for ( int k = 0; k < KA; ++k )
         {
            if ( k >= K ) continue;
            const float d = diff_norm(xv.x, xv.y, mu0[k], mu1[k]);
            if ( min_k == -1 || d < min_d )
            {
               min_k = k;
               min_d = d;
            }
         }
         yb[i * TILE] = (int8_t)min_k;
#pragma unroll UF
         for ( int k = 0; k < KA; ++k )
         {
            if ( k >= K ) continue;
            if ( k == min_k )
            {
               s0[k] += xv.x;
               s1[k] += xv.y;
               nk[k]++;
            }
         }
      }
      float n0[KA], n1[KA];
      bool means_same = true;
#pragma unroll UF
      for ( int k = 0; k < KA; ++k )
      {
         if ( k >= K ) continue;
         const float sc = 1.0f / nk[k];
         n0[k] = s0[k] * sc;
         n1[k] = s1[k] * sc;
         means_same = means_same && __float_as_uint(n0[k]) == __float_as_uint(mu0[k])
                      && __float_as_uint(n1[k]) == __float_as_uint(mu1[k]) && nk[k] == nprev[k];
      }
      bool same;
      if ( first )
      {
         same = nk[0] == N;
      }
      else if ( means_same )
      {
         same = true;
         same = labels_equal(ya, yb, N);
      }
      else
      {
         same = false;
      }
      bool done = same;
      int8_t* lab = yb;            /* converged: the unchanged assignment, means unchanged */
      if ( !same )
      {
         int8_t* tmp = ya;
         ya = yb;
         yb = tmp;
         first = false;
#pragma unroll UF
         for ( int k = 0; k < KA; ++k )
         {
            if ( k >= K ) continue;
            mu0[k] = n0[k];
            mu1[k] = n1[k];
            nprev[k] = nk[k];
         }
         done = ++t == 300;
         lab = ya;                 /* ran out: the last assignment, means updated from it */
      }
      if ( !done ) continue;
      running = false;
      if ( !pending )
      {
         int8_t* tmp = pl;
         pl = lab;
         if ( lab == ya ) ya = tmp; else yb = tmp;
#pragma unroll UF
         for ( int k = 0; k < KA; ++k )
         {
            if ( k >= K ) continue;
            pm0[k] = mu0[k];
            pm1[k] = mu1[k];
         }
         pending = true;
      }
      else
      {
         held = true;
         hl = lab;
      }
   }
   return bestLogL;
}

#ifndef KINC_KMEANS_LANE_INDEPENDENT
#define KINC_KMEANS_LANE_INDEPENDENT 0
#endif

/*
 * KMeans::fit (src/core/pairwise_kmeans.cpp:12-99) for one lane's pair with K
 * clusters: 10 initialisations (means drawn from rand()), each up to 300
 * Lloyd iterations until no label changes, the one with the largest
 * log-likelihood kept.  Each lane walks its own (init, iteration) sequence:
 * a lane whose initialisation has converged starts its next one while the
 * other lanes of the warp are still iterating, so a warp costs the largest
 * total of iterations over its lanes rather than the sum over inits of the
 * largest count.  The arithmetic of every lane is unchanged.
 */
template <int KT>
__device__ float kmeans_fit(const float2* X, int8_t*& cur, int8_t*& nxt, int8_t*& best, int N, int Kr,
                            LaneRng& rng, unsigned long long& units)
{
#if !KINC_KMEANS_LANE_INDEPENDENT
   return kmeans_fit_inits_in_step<KT>(X, cur, nxt, best, N, Kr, rng, units);
#else
   const int K = (KINC_STATIC_K && KT > 0) ? KT : Kr;
   constexpr int KA = KT > 0 ? KT : 64;
   constexpr int UF = KT > 0 ? KT : 1;
   float bestLogL = -INFINITY;
   if ( rng.mode == 1 ) rng.lcg = 1;
   float mu0[KA], mu1[KA];
   int8_t* ya = cur;     /* labels of the previous iteration */
   int8_t* yb = nxt;     /* labels being assigned */
   bool first = true;    /* ya is the all-zero initial vector, not yet written */
   bool fresh = true;    /* an initialisation is to be drawn */
   int t = 0;
   int init = 0;
   while ( init < 10 )
   {
      if ( fresh )
      {
#pragma unroll UF
         for ( int k = 0; k < KA; ++k )
         {
            if ( k >= K ) continue;
            const int ii = rng.next() % N;
            const float2 xv = X[ii * TILE];
            mu0[k] = xv.x;
            mu1[k] = xv.y;
         }
         ya = cur;
         yb = nxt;
         first = true;
         fresh = false;
         t = 0;
      }

      /* one Lloyd iteration: assign, compare with the previous labels, sum the new means */
      units += (unsigned long long)N * K;
      bool same = true;
      float s0[KA], s1[KA];
      int nk[KA];
#pragma unroll UF
      for ( int k = 0; k < KA; ++k )
      {
         if ( k >= K ) continue;
         s0[k] = 0.f; s1[k] = 0.f; nk[k] = 0;
      }
      float2 xn = X[0];
      for ( int i = 0; i < N; ++i )
      {
         const float2 xv = xn;
         if ( i + 1 < N ) xn = X[(i + 1) * TILE];
         if ( KINC_PREFETCH > 0 && i + KINC_PREFETCH < N )
         {
            prefetch_l2(&X[(i + KINC_PREFETCH) * TILE]);
            if ( !first ) prefetch_l2(&ya[(i + KINC_PREFETCH) * TILE]);
         }
         int min_k = -1;
         float min_d = 0.f;
#pragma unroll UF
         for ( int k = 0; k < KA; ++k )
         {
            if ( k >= K ) continue;
            const float d = diff_norm(xv.x, xv.y, mu0[k], mu1[k]);
            if ( min_k == -1 || d < min_d )
            {
               min_k = k;
               min_d = d;
            }
         }
         yb[i * TILE] = (int8_t)min_k;
         const int8_t prev = first ? (int8_t)0 : ya[i * TILE];
         same = same && (prev == (int8_t)min_k);
#pragma unroll UF
         for ( int k = 0; k < KA; ++k )
         {
            if ( k >= K ) continue;
            if ( k == min_k )
            {
               s0[k] += xv.x;
               s1[k] += xv.y;
               nk[k]++;
            }
         }
      }
      bool done = same;
      if ( !same )
      {
         int8_t* tmp = ya;
         ya = yb;
         yb = tmp;
         first = false;
#pragma unroll UF
         for ( int k = 0; k < KA; ++k )
         {
            if ( k >= K ) continue;
            const float sc = 1.0f / nk[k];
            mu0[k] = s0[k] * sc;
            mu1[k] = s1[k] * sc;
         }
         done = ++t == 300;
      }
      if ( !done ) continue;

      /* the labels: the unchanged assignment (in yb) if converged, else the last one (ya);
       * computeLogLikelihood: one accumulator, cluster-major order */
      int8_t* lab = same ? yb : ya;
      float S = 0.f;
      for ( int k = 0; k < K; ++k )
      {
         float c0 = 0.f, c1 = 0.f;
#pragma unroll UF
         for ( int kk = 0; kk < KA; ++kk )
         {
            if ( kk >= K ) continue;
            if ( kk == k ) { c0 = mu0[kk]; c1 = mu1[kk]; }
         }
         for ( int i = 0; i < N; ++i )
         {
            if ( lab[i * TILE] != k ) continue;
            const float2 xv = X[i * TILE];
            const float d = diff_norm(xv.x, xv.y, c0, c1);
            S += d * d;
         }
      }
      const float logL = -S;
      /* keep the buffers distinct: cur/nxt are this run's, best the kept one */
      if ( bestLogL < logL )
      {
         bestLogL = logL;
         int8_t* old = best;
         best = lab;
         cur = (lab == cur) ? old : cur;
         nxt = (lab == nxt) ? old : nxt;
      }
      ++init;
      fresh = true;
   }
   return bestLogL;
#endif
}

} /* namespace kinc */
