/*
 * sim_kernel.cuh -- the per-pair Similarity kernel, specialised by
 * clustering method (CLUS: 0 none, 1 GMM, 2 K-means, 3 GMM as KINC's OpenCL
 * kernels compute it, for rand_mode 1) and by the largest
 * cluster count compiled with static register arrays (KS = 3 or 5: every
 * fit, whatever its K <= KS, runs the same code with its per-component state
 * in registers, the host picks KS >= maxclus; KS = 0: the generic
 * local-memory form for any maxclus <= 64).
 * Each specialisation is instantiated in its own translation unit
 * (sim_none.cu, sim_gmm.cu, sim_kmeans.cu) so the register budget of one
 * does not constrain the others.  One CTA of 16 warps per SM (a persistent
 * grid), 128 registers per thread; warps take 32-pair tiles from a counter in
 * global memory, together per CTA round for GMM and no clustering (so the
 * SM's warps run the same code region at a time), one at a time for K-means.
 */
#pragma once

#include "sim_device.cuh"

namespace kinc {

#ifndef KINC_WARPS_PER_BLOCK
#define KINC_WARPS_PER_BLOCK 16
#endif
constexpr int WARPS_PER_BLOCK = KINC_WARPS_PER_BLOCK;
/* KINC_CTA_ROUNDS: the warps of a CTA take their tiles together and wait for
 * one another before the next round, so they run the same code region at the
 * same time (a warp that drifts into another fit or phase evicts the others'
 * instructions) */
#ifndef KINC_CTA_ROUNDS
#define KINC_CTA_ROUNDS 3           /* bit c set: rounds for clusmethod c (0 none, 1 gmm, 2 kmeans) */
#endif
#ifndef KINC_MIN_BLOCKS
#define KINC_MIN_BLOCKS (16 / KINC_WARPS_PER_BLOCK)
#endif
/* GMM takes 20-warp CTAs: at 96 registers (spilling a few hundred bytes to L1) the fits' fixed-
 * latency chains hide behind 25 % more warps, which beats 16 warps at 128 registers by 16 % */
#ifndef KINC_GMM_WARPS_PER_BLOCK
#define KINC_GMM_WARPS_PER_BLOCK 20
#endif

/* warps per CTA at most for clustering method CLUS (3: GMM in the OpenCL worker's form); the
 * kernel's register budget follows from it, and the host sizes grids and scratch slots by it */
template <int CLUS>
__host__ __device__ constexpr int kernel_warps()
{
   return (CLUS == 1 || CLUS == 3) ? KINC_GMM_WARPS_PER_BLOCK : WARPS_PER_BLOCK;
}

template <int CLUS>
__host__ __device__ constexpr int kernel_min_blocks()
{
   return (CLUS == 1 || CLUS == 3) ? (KINC_GMM_WARPS_PER_BLOCK <= 16 ? 16 / KINC_GMM_WARPS_PER_BLOCK : 1)
                                   : KINC_MIN_BLOCKS;
}

/* What the reference left in its packed array at position i by pair c: the
 * i-th usable sample (0-based) of c.  Reads come with increasing i for the
 * same or an earlier pair, so the word scan resumes where the last one ended
 * while c is unchanged. */
struct PackedCursor
{
   int64_t c = -1;
   int w = 0;          /* current mask word */
   int before = 0;     /* usable samples in words < w */
   int32_t x = 0, y = 0;

   __device__ float2 at(const DevParams& P, const DevData& D, int64_t pc, int i)
   {
      if ( pc != c )
      {
         c = pc;
         w = 0;
         before = 0;
         pair_xy(pc, x, y);
      }
      const uint32_t* mx = D.umask + (size_t)x * P.W;
      const uint32_t* my = D.umask + (size_t)y * P.W;
      for ( ; w < P.W; ++w )
      {
         uint32_t m = mx[w] & my[w];
         const int cnt = __popc(m);
         if ( i < before + cnt )
         {
            for ( int r = 0; r < i - before; ++r ) m &= m - 1;
            const int s = w * 32 + (__ffs(m) - 1);
            return make_float2(D.gem[(size_t)x * P.S + s], D.gem[(size_t)y * P.S + s]);
         }
         before += cnt;
      }
      return make_float2(0.f, 0.f);
   }
};

/* the closing formula of Pearson::computeCluster (pairwise_pearson.cpp:44-51): NaN below min_samples */
__device__ __forceinline__ float pearson_value(const DevParams& P, int n, float sumx, float sumy, float sumx2,
                                               float sumy2, float sumxy)
{
   if ( n >= P.min_samples )
   {
      return (n * sumxy - sumx * sumy) / sqrtf((n * sumx2 - sumx * sumx) * (n * sumy2 - sumy * sumy));
   }
   return __int_as_float(0x7fc00000);
}

/* Pearson::computeCluster for this lane's pair (pairwise_pearson.cpp:12-52); X and lbl step
 * by STR per sample (TILE: the tile's interleaved arrays, 1: a pair's own arrays). */
template <int STR = TILE>
__device__ inline float lane_pearson(const DevParams& P, const DevData& D, const DevBlock& B, const float2* X,
                                     const int8_t* lbl, int64_t p, int32_t x, int32_t y, int N, int8_t k)
{
   int n = 0;
   float sumx = 0, sumy = 0, sumx2 = 0, sumy2 = 0, sumxy = 0;
   if ( P.semantics == 0 )
   {
      /* positions i < N read the pair's own packed array at i; positions i >= N
       * read what the last earlier pair of the work block with more than i
       * usable samples left there (zero if none) */
#pragma unroll 4
      for ( int i = 0; i < N; ++i )
      {
         /* both loads unconditional (X holds N packed points), so several samples are in flight */
         const int8_t l = lbl[i * STR];
         const float2 v = X[i * STR];
         if ( l == k )
         {
            sumx += v.x; sumy += v.y; sumx2 += v.x * v.x; sumy2 += v.y * v.y; sumxy += v.x * v.y;
            ++n;
         }
      }
      /* links point strictly backwards inside the block's span [0, p - lo); anything else ends
       * the walk (defensive: the links are always written before this kernel runs) */
      const int32_t self = (int32_t)(p - B.lo);
      int32_t c = B.pg[self];
      if ( c >= self ) c = -1;
      PackedCursor cur;
      for ( int i = N; i < P.S; ++i )
      {
         if ( lbl[i * STR] != k ) continue;
         while ( c >= 0 && B.N[c] <= i )
         {
            const int32_t nxt = B.pg[c];
            c = nxt < c ? nxt : -1;
         }
         const float2 v = c >= 0 ? cur.at(P, D, B.lo + c, i) : make_float2(0.f, 0.f);
         sumx += v.x; sumy += v.y; sumx2 += v.x * v.x; sumy2 += v.y * v.y; sumxy += v.x * v.y;
         ++n;
      }
   }
   else
   {
      const float* g1 = D.gem + (size_t)x * P.S;
      const float* g2 = D.gem + (size_t)y * P.S;
      for ( int i = 0; i < P.S; ++i )
      {
         if ( lbl[i * STR] == k )
         {
            const float vx = g1[i];
            const float vy = g2[i];
            sumx += vx; sumy += vy; sumx2 += vx * vx; sumy2 += vy * vy; sumxy += vx * vy;
            ++n;
         }
      }
   }
   return pearson_value(P, n, sumx, sumy, sumx2, sumy2, sumxy);
}

/* computeBIC / computeICL (pairwise_clustering.cpp:155-172): log of the int N
 * is double, 2*logL is float, the difference is double, the result float.  The
 * OpenCL worker's GMM (OCL) evaluates them in float with log of (float)N
 * (GMM_computeBIC / GMM_computeICL, src/opencl/gmm.cl:511-530). */
template <bool OCL>
__device__ __forceinline__ float criterion_value(const DevParams& P, const DevData& D, int K, float logL, int N,
                                                 float E)
{
   const int pp = K * (1 + 2 + 2 * 2);
   if ( OCL )
   {
      float f = kinc_logf((float)N) * (float)pp - 2.0f * logL;
      if ( P.criterion == 1 ) f = f - 2.0f * E;
      return f;
   }
   double v = D.logn[N] * (double)pp - (double)(2.0f * logL);
   if ( P.criterion == 1 ) v = v - (double)(2.0f * E);
   return (float)v;
}

template <int CLUS, int KT>
__device__ __forceinline__ bool lane_fit(const DevParams& P, const float2* X, const float2* Xl, float* lpx,
                                         float* gam, int8_t*& wl, int8_t*& ya, int8_t*& yb, int8_t*& yc, int N,
                                         int K, LaneRng& rng, float& logL, float& E, unsigned long long& units,
                                         float* pbuf)
{
   if ( CLUS == 1 || CLUS == 3 )
   {
      if constexpr ( KINC_GMM_PACKED && KT >= 2 && KINC_STATIC_K && KINC_STORE_GAMMA && !KINC_STORE_LOGGAMMA &&
                     !KINC_GMM_PARAMS_SMEM )
         return gmm_fit_packed<KT, CLUS == 3>(X, lpx, gam, wl, N, rng, P.c2, logL, E, units, P.prefetch, P.neg_zero);
      else
         return gmm_fit<KT, CLUS == 3>(X, lpx, gam, wl, N, K, rng, P.c2, logL, E, units, pbuf, P.prefetch);
   }
#if KINC_KMEANS_PIPELINE
#if KINC_KMEANS_LANE_MAJOR
   /* the lane's own contiguous copy of its samples (both allocation paths provide it) */
   logL = kmeans_fit_pipelined<KT, 1>(Xl, ya, yb, wl, yc, N, K, rng, units);
#else
   logL = kmeans_fit_pipelined<KT, TILE>(X, ya, yb, wl, yc, N, K, rng, units);
#endif
#else
   logL = kmeans_fit<KT>(X, ya, yb, yc, N, K, rng, units);
#endif
   E = 0.f;
   int8_t* t = wl;   /* the best labels become the work labels */
   wl = yc;
   yc = t;
   return true;
}

/* Clustering::compute (pairwise_clustering.cpp:23-103) minus the outlier
 * passes, for this lane's pair; labels merged into lbl. */
template <int CLUS, int KS>
__device__ int lane_cluster(const DevParams& P, const DevData& D, const float2* X, float2* Xl, float* lpx,
                            float* gam, float* pbuf, int8_t* wl,
                            int8_t* ya, int8_t* yb, int8_t* yc, int8_t* lbl, int N, LaneRng& rng,
                            unsigned long long& units, unsigned long long& fits)
{
   int bestK = 0;
   if ( N < P.min_samples ) return 0;
   if ( CLUS == 2 && KINC_KMEANS_LANE_MAJOR )
      for ( int i = 0; i < N; ++i ) Xl[i] = X[i * TILE];
   float bestValue = INFINITY;
   for ( int K = P.min_k; K <= P.max_k; ++K )
   {
      float logL = 0.f, E = 0.f;
      bool ok;
      if ( !KINC_STATIC_K || KS == 0 )
         ok = lane_fit<CLUS, KS>(P, X, Xl, lpx, gam, wl, ya, yb, yc, N, K, rng, logL, E, units, pbuf);
      else if ( K == 1 ) ok = lane_fit<CLUS, 1>(P, X, Xl, lpx, gam, wl, ya, yb, yc, N, K, rng, logL, E, units, pbuf);
      else if ( K == 2 ) ok = lane_fit<CLUS, 2>(P, X, Xl, lpx, gam, wl, ya, yb, yc, N, K, rng, logL, E, units, pbuf);
      else if ( K == 3 || KS < 4 ) ok = lane_fit<CLUS, 3>(P, X, Xl, lpx, gam, wl, ya, yb, yc, N, K, rng, logL, E, units, pbuf);
      else if ( K == 4 ) ok = lane_fit<CLUS, 4>(P, X, Xl, lpx, gam, wl, ya, yb, yc, N, K, rng, logL, E, units, pbuf);
      else ok = lane_fit<CLUS, 5>(P, X, Xl, lpx, gam, wl, ya, yb, yc, N, K, rng, logL, E, units, pbuf);
      ++fits;
      if ( !ok ) continue;
      const float value = criterion_value<CLUS == 3>(P, D, K, logL, N, E);
      if ( value < bestValue )
      {
         bestK = K;
         bestValue = value;
         for ( int i = 0, j = 0; i < N; ++i )
         {
            if ( lbl[i * TILE] >= 0 )
            {
               lbl[i * TILE] = wl[j * TILE];
               ++j;
            }
         }
      }
   }
   return bestK;
}

} /* namespace kinc */

#include "sim_kmeans_pool.cuh"

namespace kinc {

template <int CLUS, int KS>
__global__ void __launch_bounds__(kernel_warps<CLUS>() * 32, kernel_min_blocks<CLUS>())
k_similarity(DevParams P, DevData D, DevScratch W, DevBlock B, int smem_sort)
{
   constexpr int CM = CLUS == 3 ? 1 : CLUS;    /* the clustering method (3: GMM, OpenCL worker's form) */
   extern __shared__ float smem[];
   const int lane = threadIdx.x & 31;
   const int warp = threadIdx.x >> 5;
   const int nwarps = blockDim.x >> 5;          /* warps per CTA: a launch-shape choice, up to kernel_warps<CLUS>() */
   const int64_t slot = blockIdx.x * (int64_t)nwarps + warp;
   const size_t col = (size_t)P.S * TILE;

   float2* X = W.X + slot * col;
   float* lpx = W.lpx + slot * col;
   float* gam = W.gam ? W.gam + slot * col * P.gam_k : nullptr;
   int8_t* lbl = W.lbl + slot * col;
   int8_t* wl = W.wl + slot * col;
   int8_t* ya = W.ya + slot * col;
   int8_t* yb = W.yb + slot * col;
   int8_t* yc = W.yc + slot * col;
   uint32_t* ring = W.rng + slot * (size_t)(RNG_WORDS * TILE);
   float* sbuf = smem_sort ? smem + (size_t)warp * P.sort_floats : W.sortbuf + slot * (size_t)P.sort_floats;
   /* GMM parameters in shared memory (KINC_GMM_PARAMS_SMEM): 7 arrays of KS x 32 floats per warp */
   float* pbuf = (CM == 1 && KINC_GMM_PARAMS_SMEM && KS > 0)
                    ? smem + (smem_sort ? (size_t)nwarps * P.sort_floats : 0) + (size_t)warp * 7 * KS * TILE
                    : nullptr;

   const int64_t ntiles = (B.size + TILE - 1) / TILE;
   const bool rounds = P.rounds != 0;         /* uniform over the launch */
   __shared__ unsigned long long round_base;
   for ( ;; )
   {
      unsigned long long t = 0;
      if ( rounds )
      {
         __syncthreads();                       /* every warp is done with the previous round */
         if ( threadIdx.x == 0 ) round_base = atomicAdd(B.tiles, (unsigned long long)nwarps);
         __syncthreads();
         const unsigned long long base = round_base;
         if ( (int64_t)base >= ntiles ) break;  /* uniform over the CTA */
         t = base + warp;
         if ( (int64_t)t >= ntiles ) continue;  /* idle this round, back to the barrier */
      }
      else
      {
         if ( lane == 0 ) t = atomicAdd(B.tiles, 1ull);
         t = __shfl_sync(0xffffffffu, t, 0);
         if ( (int64_t)t >= ntiles ) break;
      }
      const int64_t slot0 = (int64_t)t * TILE;
      const int64_t left = B.size - slot0;
      const int npairs = left < TILE ? (int)left : TILE;
      /* this lane's pair: tile slots map to pairs through the binned order */
      int64_t myp = B.start + slot0 + lane;
      if ( B.order && lane < npairs ) myp = B.start + B.order[slot0 + lane];

      /* ---- warp-cooperative: fetch, pre-outliers, rand() position, per pair */
      int myN = 0;
      for ( int j = 0; j < npairs; ++j )
      {
         const int64_t p = __shfl_sync(0xffffffffu, myp, j);
         int32_t x, y;
         pair_xy(p, x, y);
         const int n = warp_fetch(P, D, x, y, X, lbl, j, lane);
         if ( lane == j ) myN = n;
         if ( lane == 0 && n != B.N[p - B.lo] ) atomicCAS(B.status, ST_OK, ST_BAD_RANK);
         if ( CLUS != 0 )
         {
            if ( P.pre_out )
            {
               warp_mark_outliers(X, n, 0, lbl, 0, -7, sbuf, j, lane);
               warp_mark_outliers(X, n, 1, lbl, 0, -7, sbuf, j, lane);
            }
            if ( P.rand_mode == 0 && n >= P.min_samples )
            {
               const uint64_t pos = B.qpos[p - B.start] * (uint64_t)P.draws_per_pair;
               warp_rng_jump(D, pos, ring, j, lane);
            }
         }
      }
      __syncwarp();

      /* ---- lane-local: clustering */
      int K = 1;
      int32_t mx = 0, my = 0;
      if ( lane < npairs ) pair_xy(myp, mx, my);
      if ( CLUS != 0 )
      {
         unsigned long long units = 0, fits = 0;
         K = 0;
         if constexpr ( CLUS == 2 && KS > 0 )
         {
            /* the tile's runs as one pool of tasks, every lane busy until it is empty */
            LaneRng rng;
            rng.ring = ring + lane;
            rng.head = 0;
            rng.mode = P.rand_mode;
            rng.lcg = 1;
            constexpr int RS = km_record_floats<KS>();
            K = kmeans_pool<KS>(P, D, X, lbl, ya + lane, yb + lane, wl + lane, lpx + lane,
                                W.kmd + (size_t)slot * P.km_dmax * TILE, W.kmr + (size_t)slot * P.km_tmax * RS,
                                npairs, myN, rng, lane, units, fits);
         }
         else if ( lane < npairs )
         {
            LaneRng rng;
            rng.ring = ring + lane;
            rng.head = 0;
            rng.mode = P.rand_mode;
            rng.lcg = 1;
            K = lane_cluster<CLUS, KS>(P, D, X + lane,
                                       W.Xl ? W.Xl + ((size_t)slot * TILE + lane) * (size_t)P.S : nullptr,
                                       lpx + lane, gam ? gam + lane : nullptr,
                                       pbuf ? pbuf + lane : nullptr, wl + lane,
                                       ya + lane, yb + lane, yc + lane, lbl + lane, myN, rng, units, fits);
         }
         for ( int o = 16; o > 0; o >>= 1 )
         {
            units += __shfl_xor_sync(0xffffffffu, units, o);
            fits += __shfl_xor_sync(0xffffffffu, fits, o);
         }
         if ( lane == 0 && B.work )
         {
            atomicAdd(&B.work[0], units);
            atomicAdd(&B.work[1], fits);
         }
      }
      __syncwarp();

      /* ---- warp-cooperative: post-outliers */
      if ( CLUS != 0 && P.post_out )
      {
         for ( int j = 0; j < npairs; ++j )
         {
            const int Kj = __shfl_sync(0xffffffffu, K, j);
            const int nj = __shfl_sync(0xffffffffu, myN, j);
            if ( Kj > 1 )
            {
               for ( int k = 0; k < Kj; ++k )
               {
                  warp_mark_outliers(X, nj, 0, lbl, (int8_t)k, -8, sbuf, j, lane);
                  warp_mark_outliers(X, nj, 1, lbl, (int8_t)k, -8, sbuf, j, lane);
               }
            }
         }
      }

      /* ---- correlations: row [k][c], c = 0 the method asked for (or Pearson when both),
       * c = 1 Spearman when both are asked for */
      const int nc = P.ncorr;
      if ( P.corr == 0 || P.corr == 2 )
      {
         if ( lane < npairs && B.outCorr )
         {
            float* corr_row = B.outCorr + (myp - B.start) * P.max_k * nc;
            for ( int k = 0; k < P.max_k; ++k )
            {
               corr_row[k * nc] = k < K ? lane_pearson(P, D, B, X + lane, lbl + lane, myp, mx, my, myN, (int8_t)k)
                                        : __int_as_float(0x7fc00000);
            }
         }
      }
      if ( P.corr == 1 || P.corr == 2 )
      {
         const int c = P.corr == 2 ? 1 : 0;
         for ( int j = 0; j < npairs; ++j )
         {
            const int Kj = __shfl_sync(0xffffffffu, K, j);
            const int xj = __shfl_sync(0xffffffffu, mx, j);
            const int yj = __shfl_sync(0xffffffffu, my, j);
            const int64_t pj = __shfl_sync(0xffffffffu, myp, j);
            float* row = B.outCorr ? B.outCorr + (pj - B.start) * P.max_k * nc : nullptr;
            for ( int k = 0; k < P.max_k; ++k )
            {
               float r = __int_as_float(0x7fc00000);
               if ( k < Kj ) r = warp_spearman(P, D, X, lbl, xj, yj, (int8_t)k, sbuf, j, lane);
               if ( lane == 0 && row ) row[k * nc + c] = r;
            }
         }
      }

      /* ---- outputs */
      if ( lane < npairs && B.outK ) B.outK[myp - B.start] = (int8_t)K;
      if ( B.outLabels )
      {
         for ( int j = 0; j < npairs; ++j )
         {
            const int64_t pj = __shfl_sync(0xffffffffu, myp, j);
            int8_t* row = B.outLabels + (pj - B.start) * (int64_t)P.S;
            for ( int s = lane; s < P.S; s += 32 ) row[s] = lbl[s * TILE + j];
         }
      }
      __syncwarp();
   }
}

/* host-side handle of one specialisation (clus: the clustering method; ocl: the OpenCL
 * worker's GMM, CLUS 3) */
struct SimKernel
{
   const void* fn;
   int clus;
   int ks;
   bool ocl;
   int wpb;                                     /* warps per CTA at most (kernel_warps) */
};

template <int CLUS, int KS>
inline SimKernel sim_kernel_handle()
{
   return SimKernel { (const void*)&k_similarity<CLUS, KS>, CLUS == 3 ? 1 : CLUS, KS, CLUS == 3, kernel_warps<CLUS>() };
}

/* launch with P.warps warps per CTA (the host keeps it in 1..kernel_warps<CLUS>() and sizes grid,
 * smem and the scratch slots for it) */
template <int CLUS, int KS>
inline cudaError_t sim_kernel_launch(int grid, int smem, cudaStream_t st, const DevParams& P, const DevData& D,
                                     const DevScratch& W, const DevBlock& B, int smem_sort)
{
   k_similarity<CLUS, KS><<<grid, P.warps * 32, smem, st>>>(P, D, W, B, smem_sort);
   return cudaGetLastError();
}

/* defined in sim_none.cu / sim_gmm.cu / sim_kmeans.cu */
SimKernel sim_kernel_select(int clus, int max_k);
cudaError_t sim_kernel_launch_any(const SimKernel& k, int grid, int smem, cudaStream_t st, const DevParams& P,
                                  const DevData& D, const DevScratch& W, const DevBlock& B, int smem_sort);
SimKernel sim_kernel_none();
/* Pearson without clustering, one thread per pair (sim_none.cu) */
cudaError_t sim_launch_pearson_lanes(int sms, cudaStream_t st, const DevParams& P, const DevData& D,
                                     const DevBlock& B);
SimKernel sim_kernel_gmm(int max_k, bool opencl);
SimKernel sim_kernel_kmeans(int max_k);
cudaError_t sim_launch_none(const SimKernel& k, int grid, int smem, cudaStream_t st, const DevParams& P,
                            const DevData& D, const DevScratch& W, const DevBlock& B, int smem_sort);
cudaError_t sim_launch_gmm(const SimKernel& k, int grid, int smem, cudaStream_t st, const DevParams& P,
                           const DevData& D, const DevScratch& W, const DevBlock& B, int smem_sort);
cudaError_t sim_launch_kmeans(const SimKernel& k, int grid, int smem, cudaStream_t st, const DevParams& P,
                              const DevData& D, const DevScratch& W, const DevBlock& B, int smem_sort);

} /* namespace kinc */
