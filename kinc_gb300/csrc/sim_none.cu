/* Similarity kernel specialisation without clustering (clusmethod none). */
#include "sim_kernel.cuh"

#include <algorithm>

namespace kinc {

SimKernel sim_kernel_none()
{
   return sim_kernel_handle<0, 0>();
}

cudaError_t sim_launch_none(const SimKernel&, int grid, int smem, cudaStream_t st, const DevParams& P,
                            const DevData& D, const DevScratch& W, const DevBlock& B, int smem_sort)
{
   return sim_kernel_launch<0, 0>(grid, smem, st, P, D, W, B, smem_sort);
}

/*
 * Pearson without clustering (K = 1), one thread per pair, straight from the expression rows and
 * the usable-sample masks -- no compaction into scratch, no labels (rows with K <= 1 carry none).
 * Without clustering a sample position's label is 0 exactly when both genes' values are usable,
 * so Pearson::computeCluster (pairwise_pearson.cpp:12-52) reduces to: for every usable position i,
 * in order, add the point the reference reads there -- semantics 0: its packed array at i, which
 * for i < N is the pair's own i-th usable sample and for i >= N what the last earlier pair of the
 * work block with more than i usable samples left (the k_prev links; zero if none); semantics 1:
 * sample i itself.  Same sums in the same order as lane_pearson, so the same bits.
 */
__global__ void __launch_bounds__(256) k_pearson_lanes(DevParams P, DevData D, DevBlock B)
{
   const int64_t stride = (int64_t)gridDim.x * blockDim.x;
   for ( int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < B.size; q += stride )
   {
      const int64_t p = B.start + q;
      int32_t x, y;
      pair_xy(p, x, y);
      const uint32_t* mx = D.umask + (size_t)x * P.W;
      const uint32_t* my = D.umask + (size_t)y * P.W;
      const float* g1 = D.gem + (size_t)x * P.S;
      const float* g2 = D.gem + (size_t)y * P.S;
      int n = 0;
      float sumx = 0, sumy = 0, sumx2 = 0, sumy2 = 0, sumxy = 0;
      auto add = [&](float vx, float vy) {
         sumx += vx; sumy += vy; sumx2 += vx * vx; sumy2 += vy * vy; sumxy += vx * vy;
         ++n;
      };
      if ( P.semantics == 0 )
      {
         const int N = B.N[p - B.lo];
         /* positions i < N: i-th usable sample (cursor s) where position i is usable */
         int ws = 0;
         uint32_t bs = __ldg(mx) & __ldg(my);
         for ( int w = 0; w * 32 < N; ++w )
         {
            const uint32_t pos = __ldg(mx + w) & __ldg(my + w);
            const int hi = min(32, N - w * 32);
            for ( int b = 0; b < hi; ++b )
            {
               while ( bs == 0 && ws + 1 < P.W )
               {
                  ++ws;
                  bs = __ldg(mx + ws) & __ldg(my + ws);
               }
               const int s = ws * 32 + __ffs(bs) - 1;
               bs &= bs - 1;
               /* an unusable position adds +0.0, which leaves every sum as it is (a sum of floats
                * starting at +0.0 is never -0.0), so the lanes need not branch */
               const bool use = (pos >> b) & 1u;
               const float vx = use ? __ldg(g1 + s) : 0.f;
               const float vy = use ? __ldg(g2 + s) : 0.f;
               sumx += vx; sumy += vy; sumx2 += vx * vx; sumy2 += vy * vy; sumxy += vx * vy;
               n += use;
            }
         }
         /* positions i >= N: stale points of earlier pairs of the work block (as lane_pearson) */
         const int32_t self = (int32_t)(p - B.lo);
         int32_t c = B.pg[self];
         if ( c >= self ) c = -1;
         PackedCursor cur;
         for ( int w = N >> 5; w < P.W; ++w )
         {
            uint32_t pos = __ldg(mx + w) & __ldg(my + w);
            if ( w == (N >> 5) ) pos &= ~0u << (N & 31);
            while ( pos )
            {
               const int i = w * 32 + __ffs(pos) - 1;
               pos &= pos - 1;
               while ( c >= 0 && B.N[c] <= i )
               {
                  const int32_t nxt = B.pg[c];
                  c = nxt < c ? nxt : -1;
               }
               const float2 v = c >= 0 ? cur.at(P, D, B.lo + c, i) : make_float2(0.f, 0.f);
               add(v.x, v.y);
            }
         }
      }
      else
      {
         for ( int w = 0; w < P.W; ++w )
         {
            uint32_t pos = __ldg(mx + w) & __ldg(my + w);
            while ( pos )
            {
               const int i = w * 32 + __ffs(pos) - 1;
               pos &= pos - 1;
               add(__ldg(g1 + i), __ldg(g2 + i));
            }
         }
      }
      const float r = pearson_value(P, n, sumx, sumy, sumx2, sumy2, sumxy);
      if ( B.outK ) B.outK[q] = 1;
      if ( B.outCorr )
      {
         float* row = B.outCorr + q * P.max_k * P.ncorr;
         row[0] = r;
         for ( int k = 1; k < P.max_k * P.ncorr; ++k ) row[k] = __int_as_float(0x7fc00000);
      }
   }
}

cudaError_t sim_launch_pearson_lanes(int sms, cudaStream_t st, const DevParams& P, const DevData& D,
                                     const DevBlock& B)
{
   const int64_t blocks = std::min<int64_t>((B.size + 255) / 256, (int64_t)sms * 16);
   k_pearson_lanes<<<(int)std::max<int64_t>(1, blocks), 256, 0, st>>>(P, D, B);
   return cudaGetLastError();
}

} /* namespace kinc */
