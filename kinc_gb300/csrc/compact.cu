/*
 * compact.cu -- Similarity::process on the GPU (src/core/similarity.cpp:66-127):
 * the clusters of a block whose correlation passes
 * !isnan(r) && mincorr <= |r| <= maxcorr (with two correlations per cluster:
 * either of them), renumbered 0..c-1 per pair and
 * compacted, in pair order, into CMX items (x, y, c, r) and -- for pairs with
 * K > 1 -- CCM items (x, y, c, sample codes packed two per byte as the CCM
 * file stores them, sample 2i in the low nibble).  Only the kept items then
 * cross to the host.
 *
 * Three passes over chunks of CHUNK consecutive pairs: count the kept
 * clusters per chunk, exclusive-scan the counts (one block), write the items.
 */
#include "../../include/kinc_sim.h"

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

namespace {

constexpr int CHUNK = 64;          /* pairs per thread */
constexpr int THREADS = 256;

__device__ __forceinline__ bool keep(const float* r, int nc, float lo, float hi)
{
   for ( int c = 0; c < nc; ++c )
      if ( !isnan(r[c]) && lo <= fabsf(r[c]) && fabsf(r[c]) <= hi ) return true;
   return false;
}

__device__ __forceinline__ void pair_of(int64_t p, int32_t& x, int32_t& y)
{
   /* float estimate (GB300's FP64 rate is a small fraction of FP32), corrected exactly below */
   int64_t xx = (int64_t)((1.0f + sqrtf(1.0f + 8.0f * (float)p)) * 0.5f);
   while ( xx * (xx - 1) / 2 > p ) --xx;
   while ( (xx + 1) * xx / 2 <= p ) ++xx;
   x = (int32_t)xx;
   y = (int32_t)(p - xx * (xx - 1) / 2);
}

__global__ void k_compact_count(int64_t size, int max_k, int nc, const int8_t* __restrict__ K,
                                const float* __restrict__ corr, float lo, float hi,
                                unsigned long long* __restrict__ cnt_cmx, unsigned long long* __restrict__ cnt_ccm)
{
   const int64_t chunk = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
   const int64_t q0 = chunk * CHUNK;
   if ( q0 >= size ) return;
   const int64_t q1 = q0 + CHUNK < size ? q0 + CHUNK : size;
   unsigned long long a = 0, b = 0;
   for ( int64_t q = q0; q < q1; ++q )
   {
      const int k_n = K[q];
      for ( int k = 0; k < k_n; ++k )
      {
         if ( keep(corr + (q * max_k + k) * nc, nc, lo, hi) )
         {
            ++a;
            if ( k_n > 1 ) ++b;
         }
      }
   }
   cnt_cmx[chunk] = a;
   cnt_ccm[chunk] = b;
}

/* in-place exclusive scan of n counts with one block; totals at [n] */
__global__ void k_compact_scan(unsigned long long* __restrict__ v, int64_t n)
{
   __shared__ unsigned long long part[1024];
   const int t = threadIdx.x;
   const int64_t per = (n + blockDim.x - 1) / blockDim.x;
   const int64_t a = t * per;
   const int64_t b = a + per < n ? a + per : n;
   unsigned long long s = 0;
   for ( int64_t i = a; i < b; ++i ) s += v[i];
   part[t] = s;
   __syncthreads();
   if ( t == 0 )
   {
      unsigned long long run = 0;
      for ( int i = 0; i < (int)blockDim.x; ++i )
      {
         const unsigned long long x = part[i];
         part[i] = run;
         run += x;
      }
      v[n] = run;
   }
   __syncthreads();
   unsigned long long run = part[t];
   for ( int64_t i = a; i < b; ++i )
   {
      const unsigned long long x = v[i];
      v[i] = run;
      run += x;
   }
}

__global__ void k_compact_write(int64_t start, int64_t size, int max_k, int nc, int S,
                                const int8_t* __restrict__ K,
                                const int8_t* __restrict__ labels, const float* __restrict__ corr, float lo, float hi,
                                const unsigned long long* __restrict__ off_cmx,
                                const unsigned long long* __restrict__ off_ccm, int64_t cap_cmx, int64_t cap_ccm,
                                int32_t* cmx_x, int32_t* cmx_y, int8_t* cmx_c, float* cmx_r, int32_t* ccm_x,
                                int32_t* ccm_y, int8_t* ccm_c, uint8_t* ccm_nibbles)
{
   const int64_t chunk = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
   const int64_t q0 = chunk * CHUNK;
   if ( q0 >= size ) return;
   const int64_t q1 = q0 + CHUNK < size ? q0 + CHUNK : size;
   unsigned long long a = off_cmx[chunk], b = off_ccm[chunk];
   const int nb = (S + 1) / 2;
   int32_t x, y;
   pair_of(start + q0, x, y);
   for ( int64_t q = q0; q < q1; ++q )
   {
      const int k_n = K[q];
      int c1 = 0, c2 = 0;
      for ( int k = 0; k < k_n; ++k )
      {
         const float* r = corr + (q * max_k + k) * nc;
         if ( !keep(r, nc, lo, hi) ) continue;
         if ( (int64_t)a < cap_cmx && cmx_x )
         {
            cmx_x[a] = x;
            cmx_y[a] = y;
            cmx_c[a] = (int8_t)c1;
            for ( int c = 0; c < nc; ++c ) cmx_r[a * nc + c] = r[c];
         }
         ++a;
         ++c1;
         if ( k_n > 1 )
         {
            if ( (int64_t)b < cap_ccm && ccm_x && labels )
            {
               ccm_x[b] = x;
               ccm_y[b] = y;
               ccm_c[b] = (int8_t)c2;
               const int8_t* lab = labels + q * (int64_t)S;
               uint8_t* out = ccm_nibbles + b * (int64_t)nb;
               for ( int s = 0; s < S; s += 2 )
               {
                  const int8_t l0 = lab[s];
                  const int v0 = l0 >= 0 ? (k == l0) : -l0;
                  int v = v0 & 0x0F;
                  if ( s + 1 < S )
                  {
                     const int8_t l1 = lab[s + 1];
                     const int v1 = l1 >= 0 ? (k == l1) : -l1;
                     v |= (v1 << 4);
                  }
                  out[s / 2] = (uint8_t)v;
               }
            }
            ++b;
            ++c2;
         }
      }
      if ( ++y >= x )
      {
         y = 0;
         ++x;
      }
   }
}

}  // namespace

/* scratch: 2 * (ceil(size / CHUNK) + 1) counters */
size_t compact_scratch_words(int64_t size)
{
   return 2 * (size_t)((size + CHUNK - 1) / CHUNK + 1);
}

cudaError_t compact_enqueue(int64_t start, int64_t size, int max_k, int nc, int S, const int8_t* d_K,
                            const int8_t* d_labels, const float* d_corr, float lo, float hi,
                            unsigned long long* d_scratch, int64_t cap_cmx, int64_t cap_ccm, int32_t* cmx_x,
                            int32_t* cmx_y, int8_t* cmx_c, float* cmx_r, int32_t* ccm_x, int32_t* ccm_y,
                            int8_t* ccm_c, uint8_t* ccm_nibbles, unsigned long long* d_counts, cudaStream_t st)
{
   const int64_t chunks = (size + CHUNK - 1) / CHUNK;
   unsigned long long* c_cmx = d_scratch;
   unsigned long long* c_ccm = d_scratch + chunks + 1;
   const int blocks = (int)((chunks + THREADS - 1) / THREADS);
   k_compact_count<<<blocks, THREADS, 0, st>>>(size, max_k, nc, d_K, d_corr, lo, hi, c_cmx, c_ccm);
   k_compact_scan<<<1, 1024, 0, st>>>(c_cmx, chunks);
   k_compact_scan<<<1, 1024, 0, st>>>(c_ccm, chunks);
   k_compact_write<<<blocks, THREADS, 0, st>>>(start, size, max_k, nc, S, d_K, d_labels, d_corr, lo, hi, c_cmx, c_ccm,
                                               cap_cmx, cap_ccm, cmx_x, cmx_y, cmx_c, cmx_r, ccm_x, ccm_y, ccm_c,
                                               ccm_nibbles);
   cudaError_t e = cudaMemcpyAsync(d_counts, c_cmx + chunks, sizeof(unsigned long long), cudaMemcpyDeviceToDevice, st);
   if ( e == cudaSuccess )
      e = cudaMemcpyAsync(d_counts + 1, c_ccm + chunks, sizeof(unsigned long long), cudaMemcpyDeviceToDevice, st);
   if ( e == cudaSuccess ) e = cudaGetLastError();
   return e;
}
