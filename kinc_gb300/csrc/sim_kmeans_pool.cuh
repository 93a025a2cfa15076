/*
 * sim_kmeans_pool.cuh -- K-means clustering of a warp's 32-pair tile as a
 * pool of independent runs.
 *
 * KMeans::fit (src/core/pairwise_kmeans.cpp:12-99) runs 10 initialisations
 * per cluster count K, each up to 300 Lloyd iterations until no label changes,
 * and keeps the run with the largest log-likelihood; Clustering::compute
 * (src/core/pairwise_clustering.cpp:23-103) does that for K = minclus..maxclus
 * and keeps the K with the best criterion.  The runs of one pair depend on one
 * another only through the rand() stream, whose positions are known in
 * advance: run (K, init) of a pair takes its K draws at offset
 * 10 * (minclus + ... + K-1) + init * K of the pair's draws.  So the
 * 32 x (maxclus - minclus + 1) x 10 runs of a tile are independent tasks.
 * Every lane takes the next task as soon as its current one has converged,
 * so the warp's lanes stay busy until the pool is empty (lanes of the
 * one-pair-per-lane form idle while the slowest pair of the tile iterates).
 *
 * Phase A runs the Lloyd iterations of the tasks and records, per task, the
 * means its final labels were assigned with and its final means (they differ
 * when the run stops at 300 iterations, after one more mean update).  Phase B
 * re-derives each task's final labels from those means (the assignment is a
 * deterministic function of them) and computes computeLogLikelihood
 * (pairwise_kmeans.cpp:106-127) in its order -- one accumulator, cluster-major
 * -- 32 tasks at a time in lockstep.  Phase C picks, per pair and K, the first
 * initialisation with the largest log-likelihood and the K by the criterion,
 * and merges that run's labels into the pair's sample labels.  Every value is
 * computed by the reference's operation sequence, so the results are those of
 * the serial code.
 */
#pragma once

#include "sim_device.cuh"

namespace kinc {

/* floats per task record: assignment means (2K), final means (2K), log-likelihood */
template <int KT>
__host__ __device__ constexpr int km_record_floats()
{
   return 4 * KT + 1;
}

/* draws of one pair for K = kmin..kmax (10 initialisations x K each) */
__host__ __device__ inline int km_draws_per_pair(int kmin, int kmax)
{
   return 10 * (kmax * (kmax + 1) / 2 - (kmin - 1) * kmin / 2);
}

/* offset of run (K, init) in a pair's draws */
__device__ __forceinline__ int km_draw_offset(int kmin, int K, int init)
{
   return 10 * ((K - 1) * K / 2 - (kmin - 1) * kmin / 2) + init * K;
}

/* label of x under means (m0, m1)[0..K): the reference's first-minimum rule */
template <int KT>
__device__ __forceinline__ int km_assign(float x0, float x1, const float* m0, const float* m1, int K, float& min_d)
{
   int min_k = -1;
   min_d = 0.f;
#pragma unroll
   for ( int k = 0; k < KT; ++k )
   {
      if ( k >= K ) continue;
      const float d = diff_norm(x0, x1, m0[k], m1[k]);
      if ( min_k == -1 || d < min_d )
      {
         min_k = k;
         min_d = d;
      }
   }
   return min_k;
}

/* a task id -> (pair lane, K, init); tasks are ordered by K descending (longest first) */
struct KmTask
{
   int j, K, init;
};

/* position of the n-th (0-based) set bit of m */
__device__ __forceinline__ int km_nth_bit(unsigned m, int n)
{
   for ( int i = 0; i < n; ++i ) m &= m - 1u;
   return __ffs((int)m) - 1;
}

__device__ __forceinline__ KmTask km_decode(int t, int kmax, unsigned qmask, int nq)
{
   const int per_k = 10 * nq;
   KmTask d;
   d.K = kmax - t / per_k;
   const int rem = t % per_k;
   d.init = rem / nq;
   d.j = km_nth_bit(qmask, rem % nq);
   return d;
}

/* the index of task (j-th qualifying pair jj, K, init) */
__device__ __forceinline__ int km_task_index(int kmax, int K, int init, int jj, int nq)
{
   return (kmax - K) * 10 * nq + init * nq + jj;
}

/*
 * K-means for the tile: returns K for this lane's pair (0 when it has fewer than min_samples
 * usable samples) and merges the chosen run's labels into lbl.  X, lbl: the tile's interleaved
 * [S][32] arrays; ya, yb, wl: this lane's interleaved label columns; dbuf: this lane's float
 * column; draws: the tile's [draws][32] table; rec: the tile's task records.
 */
template <int KT>
__device__ int kmeans_pool(const DevParams& P, const DevData& D, const float2* X, int8_t* lbl, int8_t* ya,
                           int8_t* yb, int8_t* wl, float* dbuf, int32_t* draws, float* rec, int npairs, int myN,
                           LaneRng& rng, int lane, unsigned long long& units, unsigned long long& fits)
{
   constexpr int RS = km_record_floats<KT>();
   const int kmin = P.min_k, kmax = P.max_k;
   const int nK = kmax - kmin + 1;
   const bool qual = lane < npairs && myN >= P.min_samples;
   const int pd = P.prefetch;          /* samples ahead the sweeps prefetch into L2 (0: none) */

   /* the pair's rand() draws, in the reference's order (the LCG restarts at every fit) */
   if ( qual )
   {
      int d = 0;
      for ( int K = kmin; K <= kmax; ++K )
      {
         if ( rng.mode == 1 ) rng.lcg = 1;
         for ( int init = 0; init < 10; ++init )
            for ( int k = 0; k < K; ++k, ++d ) draws[d * TILE + lane] = rng.next() % myN;
      }
      fits += (unsigned long long)nK;
   }
   const unsigned qmask = __ballot_sync(0xffffffffu, qual);
   const int nq = __popc(qmask);
   const int T = nK * 10 * nq;
   __syncwarp();

   /* ---- phase A: Lloyd iterations of the task pool */
   bool active = false;
   int tid = 0, j = 0, K = 0, N = 0, it = 0;
   bool first = true;
   float mu0[KT], mu1[KT];
   int nprev[KT];
   int next = 0;
   for ( ;; )
   {
      /* free lanes take the next tasks (decoded by every lane so the shuffles stay uniform) */
      const unsigned freem = __ballot_sync(0xffffffffu, !active);
      if ( freem && next < T )
      {
         const int want = next + __popc(freem & lanemask_lt());
         const bool take = !active && want < T;
         const KmTask c = km_decode(take ? want : 0, kmax, qmask, nq > 0 ? nq : 1);
         const int cN = __shfl_sync(0xffffffffu, myN, c.j);
         if ( take )
         {
            tid = want;
            j = c.j;
            K = c.K;
            N = cN;
            const int off = km_draw_offset(kmin, K, c.init);
#pragma unroll
            for ( int k = 0; k < KT; ++k )
            {
               if ( k >= K ) continue;
               const int ii = draws[(off + k) * TILE + j];
               const float2 xv = X[ii * TILE + j];
               mu0[k] = xv.x;
               mu1[k] = xv.y;
               nprev[k] = -1;
            }
            it = 0;
            first = true;
            active = true;
         }
         next += __popc(freem);
      }
      if ( !__any_sync(0xffffffffu, active) ) break;

      /* one Lloyd iteration of every active lane's task, samples in lockstep */
      int maxN = active ? N : 0;
      for ( int o = 16; o > 0; o >>= 1 ) maxN = max(maxN, __shfl_xor_sync(0xffffffffu, maxN, o));
      float s0[KT], s1[KT];
      int nk[KT];
#pragma unroll
      for ( int k = 0; k < KT; ++k )
      {
         s0[k] = 0.f; s1[k] = 0.f; nk[k] = 0;
      }
      const int lim = active ? N : 0;
      /* the next KM_RING samples are in flight in registers */
      float2 ring[KM_RING];
#pragma unroll
      for ( int d = 0; d < KM_RING; ++d ) ring[d] = d < lim ? X[d * TILE + j] : make_float2(0.f, 0.f);
      for ( int i = 0; i < maxN; ++i )
      {
         if ( i < lim )
         {
            const float2 xv = ring[0];
#pragma unroll
            for ( int d = 0; d + 1 < KM_RING; ++d ) ring[d] = ring[d + 1];
            if ( i + KM_RING < lim ) ring[KM_RING - 1] = X[(i + KM_RING) * TILE + j];
            if ( pd > 0 && i + pd < lim ) prefetch_l2(&X[(i + pd) * TILE + j]);
            float md;
            const int min_k = km_assign<KT>(xv.x, xv.y, mu0, mu1, K, md);
            yb[i * TILE] = (int8_t)min_k;
#pragma unroll
            for ( int k = 0; k < KT; ++k )
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
      }
      if ( !active ) continue;
      units += (unsigned long long)N * K;
      /* "no label changed" as in kmeans_fit_inits_in_step: all in cluster 0 at the first iteration,
       * else equal means and counts and then equal label arrays */
      float n0[KT], n1[KT];
      bool means_same = true;
#pragma unroll
      for ( int k = 0; k < KT; ++k )
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
      float* r = rec + (size_t)tid * RS;
      if ( same )
      {
         /* converged: the labels were assigned with the current means, which stay */
#pragma unroll
         for ( int k = 0; k < KT; ++k )
         {
            if ( k >= K ) continue;
            r[2 * k] = mu0[k]; r[2 * k + 1] = mu1[k];
            r[2 * KT + 2 * k] = mu0[k]; r[2 * KT + 2 * k + 1] = mu1[k];
         }
         active = false;
         continue;
      }
      int8_t* tmp = ya;
      ya = yb;
      yb = tmp;
      first = false;
      if ( ++it == 300 )
      {
         /* ran out: the last labels were assigned with the current means, then the means moved */
#pragma unroll
         for ( int k = 0; k < KT; ++k )
         {
            if ( k >= K ) continue;
            r[2 * k] = mu0[k]; r[2 * k + 1] = mu1[k];
            r[2 * KT + 2 * k] = n0[k]; r[2 * KT + 2 * k + 1] = n1[k];
         }
         active = false;
         continue;
      }
#pragma unroll
      for ( int k = 0; k < KT; ++k )
      {
         if ( k >= K ) continue;
         mu0[k] = n0[k];
         mu1[k] = n1[k];
         nprev[k] = nk[k];
      }
   }
   __syncwarp();

   /* ---- phase B: log-likelihoods, 32 tasks at a time */
   for ( int b = 0; b < T; b += TILE )
   {
      const int t = b + lane;
      const bool valid = t < T;
      const KmTask c = km_decode(valid ? t : 0, kmax, qmask, nq > 0 ? nq : 1);
      const int cN = __shfl_sync(0xffffffffu, myN, c.j);
      const int lim = valid ? cN : 0;
      int maxN = lim;
      for ( int o = 16; o > 0; o >>= 1 ) maxN = max(maxN, __shfl_xor_sync(0xffffffffu, maxN, o));
      float a0[KT], a1[KT], f0[KT], f1[KT];
      float* r = rec + (size_t)(valid ? t : 0) * RS;
#pragma unroll
      for ( int k = 0; k < KT; ++k )
      {
         a0[k] = 0.f; a1[k] = 0.f; f0[k] = 0.f; f1[k] = 0.f;
         if ( valid && k < c.K )
         {
            a0[k] = r[2 * k]; a1[k] = r[2 * k + 1];
            f0[k] = r[2 * KT + 2 * k]; f1[k] = r[2 * KT + 2 * k + 1];
         }
      }
      /* the final labels and each sample's distance to its cluster's final mean */
      float2 ring[KM_RING];
#pragma unroll
      for ( int d = 0; d < KM_RING; ++d ) ring[d] = d < lim ? X[d * TILE + c.j] : make_float2(0.f, 0.f);
      for ( int i = 0; i < maxN; ++i )
      {
         if ( i < lim )
         {
            const float2 xv = ring[0];
#pragma unroll
            for ( int d = 0; d + 1 < KM_RING; ++d ) ring[d] = ring[d + 1];
            if ( i + KM_RING < lim ) ring[KM_RING - 1] = X[(i + KM_RING) * TILE + c.j];
            if ( pd > 0 && i + pd < lim ) prefetch_l2(&X[(i + pd) * TILE + c.j]);
            float md;
            const int l = km_assign<KT>(xv.x, xv.y, a0, a1, c.K, md);
            float c0 = 0.f, c1 = 0.f;
#pragma unroll
            for ( int k = 0; k < KT; ++k )
            {
               if ( k == l ) { c0 = f0[k]; c1 = f1[k]; }
            }
            ya[i * TILE] = (int8_t)l;
            dbuf[i * TILE] = diff_norm(xv.x, xv.y, c0, c1);
         }
      }
      /* computeLogLikelihood: one accumulator, cluster by cluster in sample order */
      float S = 0.f;
      for ( int k = 0; k < kmax; ++k )
      {
         const int klim = k < c.K ? lim : 0;
         /* label and distance of sample i+1 loaded (unconditionally, both written above for i < lim)
          * while sample i is added */
         int8_t ln = klim > 0 ? ya[0] : (int8_t)-1;
         float dn = klim > 0 ? dbuf[0] : 0.f;
         for ( int i = 0; i < maxN; ++i )
         {
            if ( i < klim )
            {
               const int8_t l = ln;
               const float d = dn;
               if ( i + 1 < klim )
               {
                  ln = ya[(i + 1) * TILE];
                  dn = dbuf[(i + 1) * TILE];
               }
               if ( l == k ) S += d * d;
            }
         }
      }
      if ( valid ) r[2 * KT + 2 * KT] = -S;
   }
   __syncwarp();

   /* ---- phase C: per pair, the best initialisation of each K, the K by the criterion, its labels */
   int bestK = 0;
   if ( qual )
   {
      const int jj = __popc(qmask & ((1u << lane) - 1u));
      float bestValue = INFINITY;
      int bestInit = -1;
      for ( int Kc = kmin; Kc <= kmax; ++Kc )
      {
         float bestL = -INFINITY;
         int bi = -1;
         for ( int init = 0; init < 10; ++init )
         {
            const float l = rec[(size_t)km_task_index(kmax, Kc, init, jj, nq) * RS + 4 * KT];
            if ( bestL < l )
            {
               bestL = l;
               bi = init;
            }
         }
         const float value = criterion_value<false>(P, D, Kc, bestL, myN, 0.f);
         if ( value < bestValue )
         {
            bestValue = value;
            bestK = Kc;
            bestInit = bi;
         }
      }
      if ( bestK > 0 && bestInit >= 0 )
      {
         const float* r = rec + (size_t)km_task_index(kmax, bestK, bestInit, jj, nq) * RS;
         float a0[KT], a1[KT];
#pragma unroll
         for ( int k = 0; k < KT; ++k )
         {
            a0[k] = k < bestK ? r[2 * k] : 0.f;
            a1[k] = k < bestK ? r[2 * k + 1] : 0.f;
         }
         for ( int i = 0; i < myN; ++i )
         {
            const float2 xv = X[i * TILE + lane];
            float md;
            wl[i * TILE] = (int8_t)km_assign<KT>(xv.x, xv.y, a0, a1, bestK, md);
         }
         /* the label merge of Clustering::compute: sample positions i < N with a label >= 0 */
         for ( int i = 0, q = 0; i < myN; ++i )
         {
            if ( lbl[i * TILE + lane] >= 0 )
            {
               lbl[i * TILE + lane] = wl[q * TILE];
               ++q;
            }
         }
      }
   }
   __syncwarp();
   return bestK;
}

} /* namespace kinc */
