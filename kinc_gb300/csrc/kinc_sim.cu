/*
 * kinc_sim.cu -- the GB300 Similarity worker behind include/kinc_sim.h.
 *
 * One context = one expression matrix resident in HBM plus the per-gene
 * usable-sample bitmasks, the glibc rand() jump table and the buffers of one
 * device block of pairs.  A device block runs as a short stream-ordered
 * sequence of kernels:
 *   k_count     usable-sample count N of every pair (popcount of two masks)
 *   k_scan_*    exclusive prefix of "N >= minsamp" -> each pair's position on
 *               the rand() stream (a serial KINC process draws rand() only for
 *               pairs that reach the clustering loop)
 *   k_prev      previous pair with a larger N inside the same 32768-pair work
 *               block (what the reference's stale packed-array reads see)
 *   k_similarity  the per-pair work (sim_device.cuh)
 * Replaces Similarity::OpenCL::{initialize, Worker::Worker, Worker::execute}
 * (src/core/similarity_opencl.cpp:34-70, src/core/similarity_opencl_worker.cpp:50-271).
 */
#include "../../include/kinc_sim.h"
#include "sim_internal.h"
#include "sim_kernel.cuh"
#include "pearson_tc.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <mutex>
#include <string>
#include <vector>

#include <sys/stat.h>

using namespace kinc;

/* compact.cu */
size_t compact_scratch_words(int64_t size);
cudaError_t compact_enqueue(int64_t start, int64_t size, int max_k, int ncorr, int S, const int8_t* d_K,
                            const int8_t* d_labels, const float* d_corr, float lo, float hi,
                            unsigned long long* d_scratch, int64_t cap_cmx, int64_t cap_ccm, int32_t* cmx_x,
                            int32_t* cmx_y, int8_t* cmx_c, float* cmx_r, int32_t* ccm_x, int32_t* ccm_y,
                            int8_t* ccm_c, uint8_t* ccm_nibbles, unsigned long long* d_counts, cudaStream_t st);

namespace {

constexpr int SCAN_THREADS = 1024;

/* ================================================================ kernels */

__global__ void k_masks(const float* __restrict__ gem, int32_t G, int32_t S, int32_t W, float min_expr,
                        uint32_t* __restrict__ umask)
{
   const int64_t w_total = (int64_t)G * W;
   for ( int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < w_total;
         t += (int64_t)gridDim.x * blockDim.x )
   {
      const int64_t g = t / W;
      const int w = (int)(t % W);
      uint32_t m = 0;
      for ( int b = 0; b < 32; ++b )
      {
         const int s = w * 32 + b;
         if ( s < S )
         {
            const float v = gem[g * S + s];
            if ( !isnan(v) && !(v < min_expr) ) m |= 1u << b;
         }
      }
      umask[t] = m;
   }
}

__device__ __forceinline__ int pair_count(const uint32_t* __restrict__ umask, int W, int64_t p)
{
   int32_t x, y;
   pair_xy(p, x, y);
   const uint32_t* mx = umask + (size_t)x * W;
   const uint32_t* my = umask + (size_t)y * W;
   int n = 0;
   for ( int w = 0; w < W; ++w ) n += __popc(mx[w] & my[w]);
   return n;
}

/* N for pairs [lo, lo + count) */
__global__ void k_count(const uint32_t* __restrict__ umask, int W, int64_t lo, int64_t count,
                        int32_t* __restrict__ N)
{
   for ( int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < count;
         t += (int64_t)gridDim.x * blockDim.x )
   {
      N[t] = pair_count(umask, W, lo + t);
   }
}

/* number of pairs in [0, end) with N >= min_samples, added into *acc */
__global__ void k_count_qualifying(const uint32_t* __restrict__ umask, int W, int64_t end, int min_samples,
                                   unsigned long long* acc)
{
   __shared__ unsigned long long sh[32];
   unsigned long long c = 0;
   for ( int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < end;
         t += (int64_t)gridDim.x * blockDim.x )
   {
      c += pair_count(umask, W, t) >= min_samples;
   }
   for ( int o = 16; o > 0; o >>= 1 ) c += __shfl_xor_sync(0xffffffffu, c, o);
   if ( (threadIdx.x & 31) == 0 ) sh[threadIdx.x >> 5] = c;
   __syncthreads();
   if ( threadIdx.x < 32 )
   {
      c = threadIdx.x < blockDim.x / 32 ? sh[threadIdx.x] : 0;
      for ( int o = 16; o > 0; o >>= 1 ) c += __shfl_xor_sync(0xffffffffu, c, o);
      if ( threadIdx.x == 0 ) atomicAdd(acc, c);
   }
}

/* block-wide exclusive scan of one value per thread (blockDim.x == SCAN_THREADS) */
__device__ unsigned long long block_exclusive_scan(unsigned long long v, unsigned long long* total)
{
   __shared__ unsigned long long warp_sums[SCAN_THREADS / 32];
   const int lane = threadIdx.x & 31;
   const int warp = threadIdx.x >> 5;
   unsigned long long incl = v;
   for ( int o = 1; o < 32; o <<= 1 )
   {
      const unsigned long long n = __shfl_up_sync(0xffffffffu, incl, o);
      if ( lane >= o ) incl += n;
   }
   if ( lane == 31 ) warp_sums[warp] = incl;
   __syncthreads();
   if ( warp == 0 )
   {
      unsigned long long ws = lane < SCAN_THREADS / 32 ? warp_sums[lane] : 0;
      for ( int o = 1; o < 32; o <<= 1 )
      {
         const unsigned long long n = __shfl_up_sync(0xffffffffu, ws, o);
         if ( lane >= o ) ws += n;
      }
      warp_sums[lane] = ws;
   }
   __syncthreads();
   const unsigned long long before = warp == 0 ? 0 : warp_sums[warp - 1];
   if ( total ) *total = warp_sums[SCAN_THREADS / 32 - 1];
   __syncthreads();
   return before + incl - v;
}

/* per scan block: number of qualifying pairs among its SCAN_THREADS pairs */
__global__ void k_scan_sums(const int32_t* __restrict__ N, int64_t offset, int64_t count, int min_samples,
                            unsigned long long* __restrict__ bsum)
{
   const int64_t t = blockIdx.x * (int64_t)SCAN_THREADS + threadIdx.x;
   const unsigned long long f = (t < count && N[offset + t] >= min_samples) ? 1ull : 0ull;
   unsigned long long total;
   block_exclusive_scan(f, &total);
   if ( threadIdx.x == 0 ) bsum[blockIdx.x] = total;
}

/* exclusive scan of the block sums (one block, several passes), plus the base */
__global__ void k_scan_blocks(unsigned long long* __restrict__ bsum, int nblocks,
                              unsigned long long* __restrict__ qbase)
{
   unsigned long long carry = *qbase;
   for ( int base = 0; base < nblocks; base += SCAN_THREADS )
   {
      const int i = base + threadIdx.x;
      const unsigned long long v = i < nblocks ? bsum[i] : 0ull;
      unsigned long long total;
      const unsigned long long ex = block_exclusive_scan(v, &total);
      if ( i < nblocks ) bsum[i] = carry + ex;
      carry += total;
   }
   if ( threadIdx.x == 0 ) *qbase = carry;   /* qualifying pairs before the next block */
}

__global__ void k_scan_apply(const int32_t* __restrict__ N, int64_t offset, int64_t count, int min_samples,
                             const unsigned long long* __restrict__ boff, uint64_t* __restrict__ qpos)
{
   const int64_t t = blockIdx.x * (int64_t)SCAN_THREADS + threadIdx.x;
   const unsigned long long f = (t < count && N[offset + t] >= min_samples) ? 1ull : 0ull;
   const unsigned long long ex = block_exclusive_scan(f, nullptr);
   if ( t < count ) qpos[t] = boff[blockIdx.x] + ex;
}

/* previous pair (same 32768-pair work block) with a strictly larger N: a CTA
 * builds a max-tree of its work block's N in shared memory (internal
 * nodes 1..WB-1; leaf i is N of the block's i-th pair, -1 past its end) and
 * every pair searches it independently -- up the tree until a left sibling
 * holds a larger maximum, then down that subtree keeping to the right.  Links
 * are offsets from lo (-1 = none); lo is a work-block boundary. */
constexpr int PREV_THREADS = 1024;
constexpr int PREV_SMEM = KINC_SIM_WORK_BLOCK_SIZE * (int)sizeof(int32_t);

__global__ void __launch_bounds__(PREV_THREADS) k_prev(const int32_t* __restrict__ N, int64_t lo, int64_t end,
                                                       int32_t* __restrict__ pg, int split)
{
   constexpr int WB = KINC_SIM_WORK_BLOCK_SIZE;
   extern __shared__ int32_t tree[];
   /* `split` CTAs per work block: each builds the block's tree and answers its share of the pairs */
   const int part = (int)(blockIdx.x % split);
   const int64_t b0 = lo + (int64_t)(blockIdx.x / split) * WB;
   const int64_t n64 = end - b0 < WB ? end - b0 : WB;
   const int n = (int)n64;
   const int32_t* Nb = N + (b0 - lo);
   auto leaf = [&](int i) -> int32_t { return i < n ? Nb[i] : -1; };
   auto node = [&](int k) -> int32_t { return k >= WB ? leaf(k - WB) : tree[k]; };

   for ( int k = WB / 2 + threadIdx.x; k < WB; k += PREV_THREADS )
      tree[k] = max(leaf(2 * k - WB), leaf(2 * k + 1 - WB));
   __syncthreads();
   for ( int level = WB / 4; level >= 1; level >>= 1 )
   {
      for ( int k = level + threadIdx.x; k < 2 * level; k += PREV_THREADS ) tree[k] = max(tree[2 * k], tree[2 * k + 1]);
      __syncthreads();
   }
   const int share = (n + split - 1) / split;
   const int o_end = min(n, (part + 1) * share);
   for ( int o = part * share + threadIdx.x; o < o_end; o += PREV_THREADS )
   {
      const int32_t v = Nb[o];
      int ans = -1;
      for ( int idx = WB + o; idx > 1; idx >>= 1 )
      {
         if ( !(idx & 1) || node(idx - 1) <= v ) continue;
         int s = idx - 1;            /* the nearest range to the left with a larger N */
         while ( s < WB ) s = node(2 * s + 1) > v ? 2 * s + 1 : 2 * s;
         ans = s - WB;
         break;
      }
      pg[(b0 - lo) + o] = ans >= 0 ? (int32_t)((b0 - lo) + ans) : -1;
   }
}

/* the links of every work block of [lo, end) (lo a work-block boundary) */
cudaError_t launch_prev(const int32_t* N, int64_t lo, int64_t end, int32_t* pg, cudaStream_t st)
{
   const cudaError_t attr = cudaFuncSetAttribute(k_prev, cudaFuncAttributeMaxDynamicSharedMemorySize, PREV_SMEM);
   if ( attr != cudaSuccess ) return attr;
   const int64_t nwb = (end - 1) / KINC_SIM_WORK_BLOCK_SIZE - lo / KINC_SIM_WORK_BLOCK_SIZE + 1;
   int dev = 0, sms = 0;
   cudaGetDevice(&dev);
   cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
   /* enough CTAs for two per SM: a few work blocks split their pairs over several CTAs */
   const int split = (int)std::max<int64_t>(1, std::min<int64_t>(16, (2 * (int64_t)sms + nwb - 1) / nwb));
   k_prev<<<(int)(nwb * split), PREV_THREADS, PREV_SMEM, st>>>(N, lo, end, pg, split);
   return cudaGetLastError();
}

/* counting sort of a block's pairs by usable-sample count, largest first, so a
 * warp's 32 pairs have similar trip counts and the heaviest tiles start first */
constexpr int BIN_THREADS = 256;
constexpr int MAX_BINS = 4096;

__global__ void k_bin_hist(const int32_t* __restrict__ N, int64_t off, int64_t size, int shift, int nbins,
                           unsigned int* __restrict__ hist)
{
   __shared__ unsigned int h[MAX_BINS];
   for ( int i = threadIdx.x; i < nbins; i += blockDim.x ) h[i] = 0;
   __syncthreads();
   for ( int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < size; t += (int64_t)gridDim.x * blockDim.x )
   {
      atomicAdd(&h[N[off + t] >> shift], 1u);
   }
   __syncthreads();
   for ( int i = threadIdx.x; i < nbins; i += blockDim.x )
      if ( h[i] ) atomicAdd(&hist[i], h[i]);
}

/* exclusive scan in descending bin order (one thread; nbins <= 4096) */
__global__ void k_bin_offsets(unsigned int* __restrict__ hist, int nbins)
{
   if ( threadIdx.x != 0 ) return;
   unsigned int run = 0;
   for ( int b = nbins - 1; b >= 0; --b )
   {
      const unsigned int c = hist[b];
      hist[b] = run;
      run += c;
   }
}

__global__ void k_bin_scatter(const int32_t* __restrict__ N, int64_t off, int64_t size, int shift,
                              unsigned int* __restrict__ cursor, int32_t* __restrict__ order)
{
   for ( int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < size; t += (int64_t)gridDim.x * blockDim.x )
   {
      const unsigned int pos = atomicAdd(&cursor[N[off + t] >> shift], 1u);
      order[pos] = (int32_t)t;
   }
}

/* ============================================================ host side */

struct DevBuf
{
   void* p = nullptr;
   size_t bytes = 0;
};

}  // namespace

struct kinc_sim_ctx
{
   kinc_sim_params params {};
   int32_t G = 0, S = 0, W = 0;
   DevParams dp {};
   DevData dd {};
   DevScratch ds {};
   cudaStream_t stream = nullptr;
   SimKernel kern {};
   TcState tc;                      /* tensor-core Pearson form (precision != 0) */
   bool use_tc = false;
   int grid = 0;                    /* CTAs of the current launch shape */
   int smem_bytes = 0;              /* dynamic shared memory of one CTA of the current shape */
   int smem_sort = 0;
   int smem_warp = 0;               /* dynamic shared memory per warp */
   int sms = 0;
   int64_t slots = 0;               /* warp scratch slots allocated */
   kinc_sim_launch launch {};
   char gpu_name[256] = "";
   int64_t max_block = 0;
   /* device allocations */
   float* d_gem = nullptr;
   uint32_t* d_umask = nullptr;
   double* d_logn = nullptr;
   uint32_t* d_jump = nullptr;
   uint32_t* d_rng0 = nullptr;
   int32_t* d_N = nullptr;
   int32_t* d_pg = nullptr;
   uint64_t* d_qpos = nullptr;
   unsigned long long* d_bsum = nullptr;
   unsigned long long* d_qbase = nullptr;
   unsigned long long* d_tiles = nullptr;
   unsigned long long* d_work = nullptr;
   unsigned long long* d_compact = nullptr;   /* per-chunk counters of the device process() */
   int32_t* d_order = nullptr;                /* binned tile order of the current block */
   unsigned int* d_bins = nullptr;
   int bin_shift = 0, nbins = 1;
   int* d_status = nullptr;
   int8_t* d_K = nullptr;
   int8_t* d_labels = nullptr;
   float* d_corr = nullptr;
   void* d_scratch = nullptr;
   /* host-side tracking of the rand() position held in d_qbase */
   int64_t q_valid_end = 0;
   int32_t launches = 0;
   std::string err;
};

namespace {

/* message of the calling thread's last failure that had no context (kinc_sim_create, the
 * allocation-free entry point): a fixed per-thread buffer, so threads do not race on it and
 * reporting an error allocates nothing */
constexpr size_t ERROR_CHARS = 512;
thread_local char g_create_error[ERROR_CHARS] = "";

int fail(kinc_sim_ctx* ctx, int code, const char* fmt, ...)
{
   char buf[ERROR_CHARS];
   va_list ap;
   va_start(ap, fmt);
   vsnprintf(buf, sizeof buf, fmt, ap);
   va_end(ap);
   if ( ctx ) ctx->err = buf; else memcpy(g_create_error, buf, sizeof buf);
   return code;
}

#define CK(call)                                                                                    \
   do                                                                                               \
   {                                                                                                \
      cudaError_t e_ = (call);                                                                      \
      if ( e_ != cudaSuccess )                                                                      \
         return fail(ctx, e_ == cudaErrorMemoryAllocation ? KINC_SIM_ENOMEM : KINC_SIM_ECUDA,       \
                     "%s: %s", #call, cudaGetErrorString(e_));                                      \
   } while ( 0 )

/* glibc TYPE_3 rand(): state before output 0 and the jump matrices A^(2^b). */
void glibc_rng_tables(std::vector<uint32_t>& rng0, std::vector<uint32_t>& jump)
{
   std::vector<int64_t> r(344);
   r[0] = 1;
   for ( int i = 1; i < 31; ++i )
   {
      const int64_t hi = r[i - 1] / 127773;
      const int64_t lo = r[i - 1] % 127773;
      int64_t word = 16807 * lo - 2836 * hi;
      if ( word < 0 ) word += 2147483647;
      r[i] = word;
   }
   for ( int i = 31; i < 34; ++i ) r[i] = r[i - 31];
   for ( int i = 34; i < 344; ++i ) r[i] = (int64_t)(uint32_t)((uint32_t)r[i - 31] + (uint32_t)r[i - 3]);
   rng0.resize(RNG_WORDS);
   for ( int i = 0; i < RNG_WORDS; ++i ) rng0[i] = (uint32_t)r[313 + i];

   /* A: s'[i] = s[i+1] (i < 30), s'[30] = s[0] + s[28]; row-major M[row][col] */
   const int n = RNG_WORDS;
   std::vector<uint32_t> M(n * n, 0u), T(n * n);
   for ( int i = 0; i < n - 1; ++i ) M[i * n + i + 1] = 1u;
   M[(n - 1) * n + 0] = 1u;
   M[(n - 1) * n + 28] = 1u;
   jump.assign((size_t)RNG_BITS * n * n, 0u);
   for ( int b = 0; b < RNG_BITS; ++b )
   {
      for ( int row = 0; row < n; ++row )
         for ( int c = 0; c < n; ++c ) jump[(size_t)b * n * n + c * n + row] = M[row * n + c];
      for ( int i = 0; i < n; ++i )
         for ( int j = 0; j < n; ++j )
         {
            uint32_t acc = 0;
            for ( int k = 0; k < n; ++k ) acc += M[i * n + k] * M[k * n + j];
            T[i * n + j] = acc;
         }
      M.swap(T);
   }
}

int64_t draws_per_pair(const kinc_sim_params& p)
{
   if ( p.clus_method == 0 || p.rand_mode != 0 ) return 0;
   int64_t s = 0;
   for ( int k = p.min_clusters; k <= p.max_clusters; ++k ) s += k;
   return p.clus_method == 2 ? 10 * s : s;
}

int next_pow2_host(int n)
{
   int p = 2;
   while ( p < n ) p *= 2;
   return p;
}

int validate(const kinc_sim_params* p, int32_t G, int32_t S, std::string& why)
{
   char buf[256];
   if ( G < 2 ) { snprintf(buf, sizeof buf, "genes must be >= 2 (got %d)", G); why = buf; return 0; }
   if ( S < 1 ) { snprintf(buf, sizeof buf, "samples must be >= 1 (got %d)", S); why = buf; return 0; }
   if ( p->clus_method < 0 || p->clus_method > 2 ) { why = "clus_method must be 0 (none), 1 (gmm) or 2 (kmeans)"; return 0; }
   if ( p->corr_method < 0 || p->corr_method > 2 )
   {
      why = "corr_method must be 0 (pearson), 1 (spearman) or 2 (both)";
      return 0;
   }
   if ( p->min_samples < 1 ) { why = "min_samples must be >= 1"; return 0; }
   if ( p->min_clusters < 1 || p->min_clusters > 64 ) { why = "min_clusters must be in 1..64"; return 0; }
   if ( p->max_clusters < 1 || p->max_clusters > 64 ) { why = "max_clusters must be in 1..64"; return 0; }
   if ( p->max_clusters < p->min_clusters )
   {
      why = "Minimum clusters must be less than or equal to maximum clusters.";
      return 0;
   }
   if ( p->criterion < 0 || p->criterion > 1 ) { why = "criterion must be 0 (BIC) or 1 (ICL)"; return 0; }
   if ( !(p->min_corr >= 0 && p->min_corr <= 1) || !(p->max_corr >= 0 && p->max_corr <= 1) )
   {
      why = "min_corr and max_corr must be in [0, 1]";
      return 0;
   }
   if ( p->semantics < 0 || p->semantics > 1 ) { why = "semantics must be 0 or 1"; return 0; }
   if ( p->rand_mode < 0 || p->rand_mode > 1 ) { why = "rand_mode must be 0 or 1"; return 0; }
   if ( p->precision < 0 || p->precision > 4 ) { why = "precision must be 0, 1, 2, 3 or 4"; return 0; }
   if ( p->precision != 0 && (p->clus_method != 0 || p->corr_method != 0 || p->semantics != 1) )
   {
      why = "precision TF32/3xBF16/FP32-tiled/FP16 is the pairwise-complete Pearson contraction: it needs clus_method none, "
            "corr_method pearson and semantics 1 (each sample's own values)";
      return 0;
   }
   return 1;
}

}  // namespace

/* ================================================================= C ABI */

extern "C" int kinc_sim_params_default(kinc_sim_params* p)
{
   if ( !p ) return KINC_SIM_EINVAL;
   p->clus_method = 0;
   p->corr_method = 0;
   p->min_expr = -std::numeric_limits<float>::infinity();
   p->min_samples = 30;
   p->min_clusters = 1;
   p->max_clusters = 5;
   p->criterion = 1;
   p->pre_out = 0;
   p->post_out = 0;
   p->min_corr = 0.5f;
   p->max_corr = 1.0f;
   p->ksize = 4096;
   p->semantics = 0;
   p->rand_mode = 0;
   p->precision = 0;
   return KINC_SIM_OK;
}

extern "C" const char* kinc_sim_last_error(const kinc_sim_ctx* ctx)
{
   return ctx ? ctx->err.c_str() : g_create_error;
}

extern "C" int kinc_sim_get_params(const kinc_sim_ctx* ctx, kinc_sim_params* params, int32_t* genes, int32_t* samples)
{
   if ( !ctx ) return KINC_SIM_EINVAL;
   if ( params ) *params = ctx->params;
   if ( genes ) *genes = ctx->G;
   if ( samples ) *samples = ctx->S;
   return KINC_SIM_OK;
}

extern "C" int64_t kinc_sim_total_pairs(const kinc_sim_ctx* ctx)
{
   return ctx ? (int64_t)ctx->G * (ctx->G - 1) / 2 : 0;
}

extern "C" int32_t kinc_sim_num_work_blocks(const kinc_sim_ctx* ctx)
{
   const int64_t total = kinc_sim_total_pairs(ctx);
   return (int32_t)((total + KINC_SIM_WORK_BLOCK_SIZE - 1) / KINC_SIM_WORK_BLOCK_SIZE);
}

extern "C" int64_t kinc_sim_max_device_block(const kinc_sim_ctx* ctx)
{
   return ctx ? ctx->max_block : 0;
}

extern "C" int32_t kinc_sim_last_launch_count(const kinc_sim_ctx* ctx)
{
   return ctx ? ctx->launches : 0;
}

extern "C" int kinc_sim_work_counters(kinc_sim_ctx* ctx, uint64_t* out, int reset)
{
   if ( !ctx || !out ) return KINC_SIM_EINVAL;
   CK(cudaStreamSynchronize(ctx->stream));
   unsigned long long w[4];
   CK(cudaMemcpy(w, ctx->d_work, sizeof w, cudaMemcpyDeviceToHost));
   for ( int i = 0; i < 4; ++i ) out[i] = w[i];
   if ( reset ) CK(cudaMemset(ctx->d_work, 0, sizeof w));
   return KINC_SIM_OK;
}

static void release(kinc_sim_ctx* c)
{
   void* ptrs[] = { c->d_gem, c->d_umask, c->d_logn, c->d_jump, c->d_rng0, c->d_N, c->d_pg, c->d_qpos,
                    c->d_bsum, c->d_qbase, c->d_tiles, c->d_work, c->d_compact, c->d_order, c->d_bins, c->d_status, c->d_K, c->d_labels, c->d_corr,
                    c->d_scratch };
   for ( void* p : ptrs )
      if ( p ) cudaFree(p);
   tc_release(c->tc);
   if ( c->stream ) cudaStreamDestroy(c->stream);
}

extern "C" void kinc_sim_destroy(kinc_sim_ctx* ctx)
{
   if ( !ctx ) return;
   release(ctx);
   delete ctx;
}

/* per warp slot scratch of the K-means task pool (kinc::kmeans_pool) */
struct KmPool
{
   int dmax = 0, tmax = 0, rs = 0;
   size_t bytes = 0;
};

static KmPool km_pool_sizes(const kinc_sim_params& p, const SimKernel& k)
{
   KmPool m;
   if ( p.clus_method != 2 || k.ks == 0 ) return m;
   m.dmax = km_draws_per_pair(p.min_clusters, p.max_clusters);
   m.tmax = TILE * (p.max_clusters - p.min_clusters + 1) * 10;
   m.rs = k.ks == 3 ? km_record_floats<3>() : km_record_floats<5>();
   m.bytes = (((size_t)m.dmax * TILE * sizeof(int32_t) + 255) & ~(size_t)255)
             + (((size_t)m.tmax * m.rs * sizeof(float) + 255) & ~(size_t)255);
   return m;
}

/* ---------------------------------------------------------- launch shape */

/* the shape measured best on the clustering workloads: CTAs of the kernel's full warp count (20
 * for GMM, 16 otherwise), rounds for GMM and no clustering, free-running warps for K-means, the
 * sweeps prefetching 8 samples ahead */
static kinc_sim_launch default_launch(const SimKernel& k, int clus)
{
   kinc_sim_launch l {};
   l.warps_per_cta = k.wpb;
   l.rounds = ((KINC_CTA_ROUNDS) >> clus) & 1;
   l.prefetch = 8;
   return l;
}

/* warps per CTA: 4, 8, 10, 16 or 20 that divide the kernel's warp count wpb (16: 4, 8, 16;
 * 20: 4, 10, 20) */
static bool launch_valid(const kinc_sim_launch& l, int wpb)
{
   const int nw = l.warps_per_cta;
   const bool w = (nw == 4 || nw == 8 || nw == 10 || nw == 16 || nw == 20 || nw == wpb) && nw <= wpb &&
                  wpb % nw == 0;
   const bool r = l.rounds == 0 || l.rounds == 1;
   const bool f = l.prefetch == 0 || l.prefetch == 4 || l.prefetch == 8 || l.prefetch == 16;
   return w && r && f;
}

/* the grid and shared memory of a shape: as many CTAs per SM as fit, within the warp scratch
 * slots the context holds */
static int apply_launch(kinc_sim_ctx* ctx, const kinc_sim_launch& l)
{
   if ( !launch_valid(l, ctx->kern.wpb) )
      return fail(ctx, KINC_SIM_EINVAL, "launch shape warps_per_cta %d rounds %d prefetch %d not supported",
                  l.warps_per_cta, l.rounds, l.prefetch);
   const int nw = l.warps_per_cta;
   const int smem = ctx->smem_warp * nw;
   int per_sm = 0;
   CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ctx->kern.fn, nw * 32, smem));
   per_sm = std::max(1, per_sm);
   const int64_t by_slots = ctx->slots / nw;
   const int64_t grid = std::max<int64_t>(1, std::min<int64_t>((int64_t)ctx->sms * per_sm, by_slots));
   ctx->grid = (int)grid;
   ctx->smem_bytes = smem;
   ctx->launch = l;
   ctx->dp.warps = nw;
   ctx->dp.rounds = l.rounds;
   ctx->dp.prefetch = l.prefetch;
   return KINC_SIM_OK;
}

extern "C" int kinc_sim_create(const float* gem, int32_t genes, int32_t samples, const kinc_sim_params* params,
                               kinc_sim_ctx** out)
{
   kinc_sim_ctx* ctx = nullptr;
   if ( !out ) return fail(nullptr, KINC_SIM_EINVAL, "out is NULL");
   *out = nullptr;
   if ( !gem || !params ) return fail(nullptr, KINC_SIM_EINVAL, "gem and params must not be NULL");
   std::string why;
   if ( !validate(params, genes, samples, why) ) return fail(nullptr, KINC_SIM_EINVAL, "%s", why.c_str());

   ctx = new kinc_sim_ctx();
   ctx->params = *params;
   ctx->G = genes;
   ctx->S = samples;
   ctx->W = (samples + 31) / 32;
   const int S = samples;
   const int W = ctx->W;
   auto bail = [&](int code) {
      snprintf(g_create_error, ERROR_CHARS, "%s", ctx->err.c_str());
      release(ctx);
      delete ctx;
      return code;
   };
#define CKC(call)                                                                                   \
   do                                                                                               \
   {                                                                                                \
      cudaError_t e_ = (call);                                                                      \
      if ( e_ != cudaSuccess )                                                                      \
      {                                                                                             \
         fail(ctx, e_ == cudaErrorMemoryAllocation ? KINC_SIM_ENOMEM : KINC_SIM_ECUDA, "%s: %s",    \
              #call, cudaGetErrorString(e_));                                                       \
         return bail(e_ == cudaErrorMemoryAllocation ? KINC_SIM_ENOMEM : KINC_SIM_ECUDA);           \
      }                                                                                             \
   } while ( 0 )

   int dev = 0;
   CKC(cudaGetDevice(&dev));
   cudaDeviceProp prop;
   CKC(cudaGetDeviceProperties(&prop, dev));
   CKC(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));

   /* expression matrix and masks */
   const size_t gem_bytes = (size_t)genes * S * sizeof(float);
   CKC(cudaMalloc(&ctx->d_gem, gem_bytes));
   CKC(cudaMemcpyAsync(ctx->d_gem, gem, gem_bytes, cudaMemcpyHostToDevice, ctx->stream));
   CKC(cudaMalloc(&ctx->d_umask, (size_t)genes * W * sizeof(uint32_t)));
   k_masks<<<std::max(1, std::min(65535, (int)(((int64_t)genes * W + 255) / 256))), 256, 0, ctx->stream>>>(
      ctx->d_gem, genes, S, W, params->min_expr, ctx->d_umask);
   CKC(cudaGetLastError());

   /* log(N) in double, N = 0..S (computeBIC's log of an int) */
   std::vector<double> logn(S + 1);
   for ( int n = 0; n <= S; ++n ) logn[n] = std::log((double)n);
   CKC(cudaMalloc(&ctx->d_logn, logn.size() * sizeof(double)));
   CKC(cudaMemcpyAsync(ctx->d_logn, logn.data(), logn.size() * sizeof(double), cudaMemcpyHostToDevice,
                       ctx->stream));

   std::vector<uint32_t> rng0, jump;
   glibc_rng_tables(rng0, jump);
   CKC(cudaMalloc(&ctx->d_jump, jump.size() * sizeof(uint32_t)));
   CKC(cudaMalloc(&ctx->d_rng0, rng0.size() * sizeof(uint32_t)));
   CKC(cudaMemcpyAsync(ctx->d_jump, jump.data(), jump.size() * sizeof(uint32_t), cudaMemcpyHostToDevice,
                       ctx->stream));
   CKC(cudaMemcpyAsync(ctx->d_rng0, rng0.data(), rng0.size() * sizeof(uint32_t), cudaMemcpyHostToDevice,
                       ctx->stream));

   /* device parameters */
   DevParams& dp = ctx->dp;
   dp.G = genes; dp.S = S; dp.W = W;
   dp.clus = params->clus_method; dp.corr = params->corr_method;
   dp.min_expr = params->min_expr; dp.min_samples = params->min_samples;
   dp.min_k = params->min_clusters; dp.max_k = params->max_clusters;
   dp.criterion = params->criterion; dp.pre_out = params->pre_out; dp.post_out = params->post_out;
   dp.semantics = params->semantics; dp.rand_mode = params->rand_mode;
   dp.draws_per_pair = draws_per_pair(*params);
   dp.c2 = 2 * std::log(2.0f * M_PI);
   dp.neg_zero = -0.0f;
   dp.P2 = next_pow2_host(std::max(S, 2));
   const bool need_sort = (params->clus_method != 0 && (params->pre_out || params->post_out))
                          || params->corr_method >= 1;
   dp.sort_floats = params->corr_method >= 1 ? 3 * dp.P2 : (need_sort ? dp.P2 : 0);
   dp.ncorr = params->corr_method == 2 ? 2 : 1;

   /* launch shape: sort buffers in shared memory when they fit */
   const size_t sort_bytes_warp = (size_t)dp.sort_floats * sizeof(float);
   ctx->kern = params->clus_method == 0 ? sim_kernel_none()
             : params->clus_method == 1 ? sim_kernel_gmm(params->max_clusters, params->rand_mode == 1)
                                        : sim_kernel_kmeans(params->max_clusters);
   /* GMM parameters in shared memory take the room the sort buffers would use */
   const size_t param_bytes_warp = (KINC_GMM_PARAMS_SMEM && ctx->kern.clus == 1 && ctx->kern.ks > 0)
                                      ? (size_t)7 * ctx->kern.ks * TILE * sizeof(float) : 0;
   const int wpb = ctx->kern.wpb;
   ctx->smem_sort = need_sort && param_bytes_warp == 0 && sort_bytes_warp * wpb <= 200 * 1024;
   ctx->smem_bytes = (int)((ctx->smem_sort ? sort_bytes_warp : 0) + param_bytes_warp) * wpb;
   /* opt in whenever dynamic shared memory is used: the kernel's own static words count against 48 KB too */
   if ( ctx->smem_bytes > 0 )
      CKC(cudaFuncSetAttribute(ctx->kern.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, ctx->smem_bytes));
   int per_sm = 0;
   CKC(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ctx->kern.fn, wpb * 32, ctx->smem_bytes));
   per_sm = std::max(1, per_sm);

   /* scratch: per warp slot, interleaved by lane */
   const size_t col = (size_t)S * TILE;
   dp.gam_k = (KINC_STORE_GAMMA && params->clus_method == 1)
                 ? (params->max_clusters <= 3 ? 3 : params->max_clusters <= 5 ? 5 : 0) : 0;
   /* K-means with register-resident means (up to 3 or 5 clusters) runs the tile as a task pool
    * (draws and task records per slot); beyond that, per-lane fits over a contiguous copy of the
    * lane's samples */
   const KmPool km = km_pool_sizes(*params, ctx->kern);
   dp.km_dmax = km.dmax;
   dp.km_tmax = km.tmax;
   const bool lane_major = params->clus_method == 2 && KINC_KMEANS_LANE_MAJOR && ctx->kern.ks == 0;
   const size_t slot_bytes = col * sizeof(float2) * (lane_major ? 2 : 1) + col * sizeof(float) * (1 + dp.gam_k)
                             + 5 * col + (size_t)RNG_WORDS * TILE * sizeof(uint32_t)
                             + (ctx->smem_sort ? 0 : sort_bytes_warp) + km.bytes + 256 * 10;
   size_t free_b = 0, total_b = 0;
   CKC(cudaMemGetInfo(&free_b, &total_b));
   int grid = prop.multiProcessorCount * per_sm;
   const size_t scratch_cap = free_b / 4;
   while ( grid > prop.multiProcessorCount && (size_t)grid * wpb * slot_bytes > scratch_cap )
      grid -= prop.multiProcessorCount;
   const size_t slots = (size_t)grid * wpb;
   ctx->sms = prop.multiProcessorCount;
   snprintf(ctx->gpu_name, sizeof ctx->gpu_name, "%s", prop.name);
   ctx->slots = (int64_t)slots;
   ctx->smem_warp = (int)((ctx->smem_sort ? sort_bytes_warp : 0) + param_bytes_warp);
   {
      size_t off = 0;
      auto take = [&](size_t bytes) {
         const size_t o = off;
         off += (bytes + 255) & ~(size_t)255;
         return o;
      };
      const size_t oX = take(slots * col * sizeof(float2));
      const size_t oL = take(slots * col * sizeof(float));
      const size_t oG = take(slots * col * sizeof(float) * dp.gam_k);
      const size_t oB = take(slots * col);
      const size_t oW = take(slots * col);
      const size_t oA = take(slots * col);
      const size_t oY = take(slots * col);
      const size_t oC = take(slots * col);
      const size_t oR = take(slots * RNG_WORDS * TILE * sizeof(uint32_t));
      const size_t oS = take(ctx->smem_sort ? 0 : slots * sort_bytes_warp);
      const size_t oXl = take(lane_major ? slots * col * sizeof(float2) : 0);
      const size_t oKd = take(slots * (size_t)km.dmax * TILE * sizeof(int32_t));
      const size_t oKr = take(slots * (size_t)km.tmax * km.rs * sizeof(float));
      CKC(cudaMalloc(&ctx->d_scratch, off));
      char* base = (char*)ctx->d_scratch;
      ctx->ds.X = (float2*)(base + oX);
      ctx->ds.lpx = (float*)(base + oL);
      ctx->ds.gam = dp.gam_k ? (float*)(base + oG) : nullptr;
      ctx->ds.lbl = (int8_t*)(base + oB);
      ctx->ds.wl = (int8_t*)(base + oW);
      ctx->ds.ya = (int8_t*)(base + oA);
      ctx->ds.yb = (int8_t*)(base + oY);
      ctx->ds.yc = (int8_t*)(base + oC);
      ctx->ds.rng = (uint32_t*)(base + oR);
      ctx->ds.sortbuf = ctx->smem_sort ? nullptr : (float*)(base + oS);
      ctx->ds.Xl = lane_major ? (float2*)(base + oXl) : nullptr;
      ctx->ds.kmd = km.bytes ? (int32_t*)(base + oKd) : nullptr;
      ctx->ds.kmr = km.bytes ? (float*)(base + oKr) : nullptr;
   }

   /* one device block of pairs (the tensor-core form writes no labels, so its blocks can be far larger) */
   const int64_t total = (int64_t)genes * (genes - 1) / 2;
   int64_t mb = (int64_t)1 << 22;
   while ( mb > 4096 && (size_t)mb * S > ((size_t)1 << 31) ) mb >>= 1;
   if ( params->precision != 0 ) mb = (int64_t)1 << 27;
   ctx->max_block = std::min<int64_t>(mb, std::max<int64_t>(total, 1));
   const int64_t nspan = (params->precision != 0 ? 4096 : ctx->max_block) + KINC_SIM_WORK_BLOCK_SIZE;
   const int64_t nscan = (ctx->max_block + SCAN_THREADS - 1) / SCAN_THREADS;
   CKC(cudaMalloc(&ctx->d_N, nspan * sizeof(int32_t)));
   CKC(cudaMalloc(&ctx->d_pg, nspan * sizeof(int32_t)));
   CKC(cudaMalloc(&ctx->d_qpos, (params->precision != 0 ? 4096 : ctx->max_block) * sizeof(uint64_t)));
   CKC(cudaMalloc(&ctx->d_bsum, (nscan + 1) * sizeof(unsigned long long)));
   CKC(cudaMalloc(&ctx->d_qbase, sizeof(unsigned long long)));
   CKC(cudaMalloc(&ctx->d_tiles, sizeof(unsigned long long)));
   CKC(cudaMalloc(&ctx->d_work, 4 * sizeof(unsigned long long)));
   CKC(cudaMalloc(&ctx->d_compact, compact_scratch_words(ctx->max_block) * sizeof(unsigned long long)));
   /* KINC_SIM_TILE_ORDER=natural keeps the pair order in tiles (for comparisons) */
   const char* order_env = getenv("KINC_SIM_TILE_ORDER");
   if ( params->precision == 0 && !(order_env && strcmp(order_env, "natural") == 0) )
   {
      while ( (S >> ctx->bin_shift) + 1 > MAX_BINS ) ++ctx->bin_shift;
      ctx->nbins = (S >> ctx->bin_shift) + 1;
      CKC(cudaMalloc(&ctx->d_order, ctx->max_block * sizeof(int32_t)));
      CKC(cudaMalloc(&ctx->d_bins, ctx->nbins * sizeof(unsigned int)));
   }
   CKC(cudaMemsetAsync(ctx->d_work, 0, 4 * sizeof(unsigned long long), ctx->stream));
   CKC(cudaMalloc(&ctx->d_status, sizeof(int)));
   CKC(cudaMalloc(&ctx->d_K, ctx->max_block));
   if ( params->precision == 0 ) CKC(cudaMalloc(&ctx->d_labels, (size_t)ctx->max_block * S));
   CKC(cudaMalloc(&ctx->d_corr, (size_t)ctx->max_block * params->max_clusters * dp.ncorr * sizeof(float)));
   CKC(cudaMemsetAsync(ctx->d_qbase, 0, sizeof(unsigned long long), ctx->stream));
   CKC(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
   ctx->q_valid_end = 0;

   if ( params->precision != 0 )
   {
      char msg[256] = { 0 };
      cudaError_t e = tc_prepare(ctx->tc, ctx->d_gem, genes, S, params->min_expr, params->precision, ctx->stream,
                                 msg, sizeof msg);
      if ( e != cudaSuccess )
      {
         fail(ctx, e == cudaErrorMemoryAllocation ? KINC_SIM_ENOMEM : KINC_SIM_ECUDA, "tensor-core set-up: %s %s",
              cudaGetErrorString(e), msg);
         return bail(e == cudaErrorMemoryAllocation ? KINC_SIM_ENOMEM : KINC_SIM_ECUDA);
      }
      ctx->use_tc = true;
   }
   ctx->dd.gem = ctx->d_gem;
   ctx->dd.umask = ctx->d_umask;
   ctx->dd.logn = ctx->d_logn;
   ctx->dd.jump = ctx->d_jump;
   ctx->dd.rng0 = ctx->d_rng0;
   if ( params->precision == 0 )
   {
      const kinc_sim_launch def = default_launch(ctx->kern, params->clus_method);
      const int rc = apply_launch(ctx, def);
      if ( rc ) return bail(rc);
   }
   CKC(cudaStreamSynchronize(ctx->stream));
   *out = ctx;
   return KINC_SIM_OK;
#undef CKC
}

/* enqueue one device block [start, start+size) into device outputs */
static int enqueue_block(kinc_sim_ctx* ctx, int64_t start, int64_t size, int8_t* d_K, int8_t* d_labels,
                         float* d_corr, cudaStream_t st)
{
   const DevParams& dp = ctx->dp;
   if ( ctx->use_tc )
   {
      int launches = 0;
      CK(tc_enqueue(ctx->tc, ctx->G, ctx->S, dp.min_samples, dp.max_k, start, size, d_K, d_corr, ctx->d_status, st,
                    &launches));
      ctx->launches += launches;
      return KINC_SIM_OK;
   }
   const int64_t end = start + size;
   const int64_t lo = (start / KINC_SIM_WORK_BLOCK_SIZE) * KINC_SIM_WORK_BLOCK_SIZE;
   const int64_t span = end - lo;
   int launches = 0;

   k_count<<<(int)std::min<int64_t>((span + 255) / 256, 65535), 256, 0, st>>>(ctx->d_umask, ctx->W, lo, span,
                                                                               ctx->d_N);
   ++launches;
   if ( dp.clus != 0 && dp.rand_mode == 0 )
   {
      if ( ctx->q_valid_end != start )
      {
         /* rand() position of a block executed out of order: count from pair 0 */
         CK(cudaMemsetAsync(ctx->d_qbase, 0, sizeof(unsigned long long), st));
         if ( start > 0 )
         {
            k_count_qualifying<<<1024, 256, 0, st>>>(ctx->d_umask, ctx->W, start, dp.min_samples,
                                                      ctx->d_qbase);
            ++launches;
         }
      }
      const int nscan = (int)((size + SCAN_THREADS - 1) / SCAN_THREADS);
      const int64_t off = start - lo;
      k_scan_sums<<<nscan, SCAN_THREADS, 0, st>>>(ctx->d_N, off, size, dp.min_samples, ctx->d_bsum);
      k_scan_blocks<<<1, SCAN_THREADS, 0, st>>>(ctx->d_bsum, nscan, ctx->d_qbase);
      k_scan_apply<<<nscan, SCAN_THREADS, 0, st>>>(ctx->d_N, off, size, dp.min_samples, ctx->d_bsum,
                                                   ctx->d_qpos);
      launches += 3;
      ctx->q_valid_end = end;
   }
   if ( (dp.corr == 0 || dp.corr == 2) && dp.semantics == 0 )
   {
      /* every Pearson run with the reference's packed-array reads needs the links */
      CK(launch_prev(ctx->d_N, lo, end, ctx->d_pg, st));
      ++launches;
   }
   /* Pearson without clustering runs one thread per pair straight from the matrix (no tiles) */
   const bool lanes = dp.clus == 0 && dp.corr == 0;
   if ( ctx->d_order && size > TILE && !lanes )
   {
      const int64_t off = start - lo;
      const int g = (int)std::min<int64_t>((size + BIN_THREADS - 1) / BIN_THREADS, 1024);
      CK(cudaMemsetAsync(ctx->d_bins, 0, ctx->nbins * sizeof(unsigned int), st));
      k_bin_hist<<<g, BIN_THREADS, 0, st>>>(ctx->d_N, off, size, ctx->bin_shift, ctx->nbins, ctx->d_bins);
      k_bin_offsets<<<1, 32, 0, st>>>(ctx->d_bins, ctx->nbins);
      k_bin_scatter<<<g, BIN_THREADS, 0, st>>>(ctx->d_N, off, size, ctx->bin_shift, ctx->d_bins, ctx->d_order);
      launches += 3;
   }
   CK(cudaMemsetAsync(ctx->d_tiles, 0, sizeof(unsigned long long), st));
   DevBlock B;
   B.start = start;
   B.size = size;
   B.lo = lo;
   B.N = ctx->d_N;
   B.pg = ctx->d_pg;
   B.qpos = ctx->d_qpos;
   B.order = (ctx->d_order && size > TILE) ? ctx->d_order : nullptr;
   B.outK = d_K;
   B.outLabels = d_labels;
   B.outCorr = d_corr;
   B.tiles = ctx->d_tiles;
   B.status = ctx->d_status;
   B.work = ctx->d_work;
   if ( lanes )
   {
      CK(sim_launch_pearson_lanes(ctx->sms, st, dp, ctx->dd, B));
   }
   else
   {
      const SimKernel& k = ctx->kern;
      cudaError_t e = k.clus == 0 ? sim_launch_none(k, ctx->grid, ctx->smem_bytes, st, dp, ctx->dd, ctx->ds, B,
                                                    ctx->smem_sort)
                    : k.clus == 1 ? sim_launch_gmm(k, ctx->grid, ctx->smem_bytes, st, dp, ctx->dd, ctx->ds, B,
                                                   ctx->smem_sort)
                                  : sim_launch_kmeans(k, ctx->grid, ctx->smem_bytes, st, dp, ctx->dd, ctx->ds, B,
                                                      ctx->smem_sort);
      CK(e);
   }
   ++launches;
   ctx->launches += launches;
   return KINC_SIM_OK;
}

static int check_range(kinc_sim_ctx* ctx, int64_t start, int64_t size)
{
   const int64_t total = kinc_sim_total_pairs(ctx);
   if ( start < 0 || size < 0 || start + size > total )
      return fail(ctx, KINC_SIM_EINVAL, "pair range [%lld, %lld) outside [0, %lld)", (long long)start,
                  (long long)(start + size), (long long)total);
   return KINC_SIM_OK;
}

int kinc_sim_status_copy_async(kinc_sim_ctx* ctx, uint64_t* dst, cudaStream_t stream)
{
   if ( !ctx || !dst ) return KINC_SIM_EINVAL;
   CK(cudaMemsetAsync(dst, 0, sizeof(uint64_t), stream));
   CK(cudaMemcpyAsync(dst, ctx->d_status, sizeof(int), cudaMemcpyDeviceToDevice, stream));
   return KINC_SIM_OK;
}

extern "C" int kinc_sim_synchronize(kinc_sim_ctx* ctx)
{
   if ( !ctx ) return KINC_SIM_EINVAL;
   CK(cudaStreamSynchronize(ctx->stream));
   int st = 0;
   CK(cudaMemcpy(&st, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost));
   if ( st != ST_OK )
   {
      CK(cudaMemset(ctx->d_status, 0, sizeof(int)));
      return fail(ctx, KINC_SIM_EKERNEL, "kernel reported status %d", st);
   }
   return KINC_SIM_OK;
}

extern "C" int kinc_sim_execute_block_device(kinc_sim_ctx* ctx, int64_t start, int64_t size, int8_t* d_K,
                                             int8_t* d_labels, float* d_corr, void* stream)
{
   if ( !ctx ) return KINC_SIM_EINVAL;
   int rc = check_range(ctx, start, size);
   if ( rc ) return rc;
   if ( size > ctx->max_block )
      return fail(ctx, KINC_SIM_EINVAL, "size %lld exceeds the device block limit %lld", (long long)size,
                  (long long)ctx->max_block);
   if ( size == 0 ) return KINC_SIM_OK;
   ctx->launches = 0;
   cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
   return enqueue_block(ctx, start, size, d_K, d_labels, d_corr, st);
}

/* ------------------------------------------------------------- autotuner */

extern "C" int kinc_sim_get_launch(const kinc_sim_ctx* ctx, kinc_sim_launch* launch)
{
   if ( !ctx || !launch ) return KINC_SIM_EINVAL;
   *launch = ctx->launch;
   return KINC_SIM_OK;
}

extern "C" int kinc_sim_set_launch(kinc_sim_ctx* ctx, const kinc_sim_launch* launch)
{
   if ( !ctx || !launch ) return KINC_SIM_EINVAL;
   if ( ctx->use_tc ) return fail(ctx, KINC_SIM_EINVAL, "the tensor-core precisions have no per-pair launch shape");
   return apply_launch(ctx, *launch);
}

namespace {

/* the cache file named in include/kinc_sim.h */
std::string tune_cache_path()
{
   if ( const char* p = getenv("KINC_TUNE_CACHE") ) return p;
   if ( const char* x = getenv("XDG_CACHE_HOME") ) return std::string(x) + "/kinc_gb300/launch.txt";
   if ( const char* h = getenv("HOME") ) return std::string(h) + "/.cache/kinc_gb300/launch.txt";
   return "";
}

std::string tune_key(const kinc_sim_ctx* ctx)
{
   const kinc_sim_params& p = ctx->params;
   char buf[400];
   snprintf(buf, sizeof buf, "clus=%d ks=%d ocl=%d corr=%d sem=%d pre=%d post=%d maxk=%d S<=%d gpu=%s sms=%d",
            p.clus_method, ctx->kern.ks, (int)ctx->kern.ocl, p.corr_method, p.semantics, p.pre_out, p.post_out,
            p.max_clusters, next_pow2_host(std::max(ctx->S, 2)), ctx->gpu_name, ctx->sms);
   for ( char* c = buf; *c; ++c )
      if ( *c == '\t' || *c == '\n' ) *c = ' ';
   return buf;
}

bool tune_cache_lookup(const std::string& key, int wpb, kinc_sim_launch& out)
{
   const std::string path = tune_cache_path();
   if ( path.empty() ) return false;
   FILE* f = fopen(path.c_str(), "r");
   if ( !f ) return false;
   char line[1024];
   bool found = false;
   while ( fgets(line, sizeof line, f) )
   {
      char* tab = strchr(line, '\t');
      if ( !tab ) continue;
      *tab = 0;
      kinc_sim_launch l {};
      if ( key == line && sscanf(tab + 1, "%d %d %d", &l.warps_per_cta, &l.rounds, &l.prefetch) == 3
           && launch_valid(l, wpb) )
      {
         out = l;          /* the last entry for a key wins */
         found = true;
      }
   }
   fclose(f);
   return found;
}

void tune_cache_store(const std::string& key, const kinc_sim_launch& l, double ms, int64_t pairs)
{
   const std::string path = tune_cache_path();
   if ( path.empty() ) return;
   /* create the directory chain of the file if needed */
   for ( size_t i = 1; i < path.size(); ++i )
   {
      if ( path[i] != '/' ) continue;
      const std::string dir = path.substr(0, i);
      mkdir(dir.c_str(), 0755);
   }
   FILE* f = fopen(path.c_str(), "a");
   if ( !f ) return;
   fprintf(f, "%s\t%d %d %d\t%.4f ms for %lld pairs\n", key.c_str(), l.warps_per_cta, l.rounds, l.prefetch, ms,
           (long long)pairs);
   fclose(f);
}

}  // namespace

static int time_launch(kinc_sim_ctx* ctx, const kinc_sim_launch& l, int64_t start, int64_t size, double& ms)
{
   int rc = apply_launch(ctx, l);
   if ( rc ) return rc;
   cudaEvent_t e0 = nullptr, e1 = nullptr;
   CK(cudaEventCreate(&e0));
   CK(cudaEventCreate(&e1));
   cudaError_t err = cudaEventRecord(e0, ctx->stream);
   rc = err == cudaSuccess ? enqueue_block(ctx, start, size, ctx->d_K, ctx->d_labels, ctx->d_corr, ctx->stream)
                           : KINC_SIM_ECUDA;
   if ( rc == KINC_SIM_OK ) err = cudaEventRecord(e1, ctx->stream);
   if ( rc == KINC_SIM_OK && err == cudaSuccess ) err = cudaEventSynchronize(e1);
   float t = 0.f;
   if ( rc == KINC_SIM_OK && err == cudaSuccess ) err = cudaEventElapsedTime(&t, e0, e1);
   cudaEventDestroy(e0);
   cudaEventDestroy(e1);
   if ( rc ) return rc;
   if ( err != cudaSuccess ) return fail(ctx, KINC_SIM_ECUDA, "autotune timing: %s", cudaGetErrorString(err));
   ms = t;
   return kinc_sim_synchronize(ctx);
}

extern "C" int kinc_sim_autotune(kinc_sim_ctx* ctx, int64_t start, int64_t size, int32_t use_cache,
                                 kinc_sim_launch* chosen, kinc_sim_tune_entry* entries, int32_t cap, int32_t* n)
{
   if ( !ctx ) return KINC_SIM_EINVAL;
   if ( n ) *n = 0;
   if ( ctx->use_tc ) return fail(ctx, KINC_SIM_EINVAL, "the tensor-core precisions have no per-pair launch shape");
   int rc = check_range(ctx, start, size);
   if ( rc ) return rc;
   size = std::min(size, ctx->max_block);
   if ( size <= 0 ) return fail(ctx, KINC_SIM_EINVAL, "autotune needs at least one pair");
   const std::string key = tune_key(ctx);
   kinc_sim_launch best = ctx->launch;
   if ( use_cache && tune_cache_lookup(key, ctx->kern.wpb, best) )
   {
      rc = apply_launch(ctx, best);
      if ( rc == KINC_SIM_OK && chosen ) *chosen = best;
      return rc;
   }
   CK(cudaStreamSynchronize(ctx->stream));
   int32_t count = 0;
   auto record = [&](const kinc_sim_launch& l, double ms) {
      if ( entries && count < cap ) entries[count] = kinc_sim_tune_entry { l, ms };
      ++count;
   };
   /* warm-up of the current shape (module load, caches), then the timed descent */
   double best_ms = 0;
   rc = time_launch(ctx, best, start, size, best_ms);
   if ( rc ) return rc;
   rc = time_launch(ctx, best, start, size, best_ms);
   if ( rc ) return rc;
   record(best, best_ms);
   const int warps_v[] = { 4, 8, 10, 16, 20 };
   const int pf_v[] = { 0, 4, 8, 16 };
   for ( int pass = 0; pass < 2; ++pass )
   {
      const kinc_sim_launch start_best = best;
      for ( int knob = 0; knob < 3; ++knob )
      {
         if ( knob == 0 && ctx->params.clus_method == 0 ) continue;   /* prefetch: the clustering sweeps only */
         /* GMM keeps its CTA rounds: free-running warps drift into different fits as a launch grows
          * longer than the timed sample, and their instructions then evict each other (a pick of
          * 20 free-running warps from a 311,296-pair sample ran 1,048,576-pair blocks at 96k
          * pairs/s against 164k in rounds) */
         if ( knob == 2 && ctx->params.clus_method == 1 ) continue;
         const int nv = knob == 0 ? 4 : knob == 1 ? 5 : 2;
         const kinc_sim_launch base = best;
         for ( int v = 0; v < nv; ++v )
         {
            kinc_sim_launch c = base;
            if ( knob == 0 ) c.prefetch = pf_v[v];
            else if ( knob == 1 ) c.warps_per_cta = warps_v[v];
            else c.rounds = v;
            if ( memcmp(&c, &base, sizeof c) == 0 || !launch_valid(c, ctx->kern.wpb) ) continue;
            double ms = 0;
            rc = time_launch(ctx, c, start, size, ms);
            if ( rc ) return rc;
            record(c, ms);
            if ( ms < best_ms )
            {
               best_ms = ms;
               best = c;
            }
         }
      }
      if ( memcmp(&best, &start_best, sizeof best) == 0 ) break;
   }
   rc = apply_launch(ctx, best);
   if ( rc ) return rc;
   if ( use_cache ) tune_cache_store(key, best, best_ms, size);
   if ( chosen ) *chosen = best;
   if ( n ) *n = count;
   return KINC_SIM_OK;
}

extern "C" int kinc_sim_execute_block(kinc_sim_ctx* ctx, int64_t start, int64_t size, int8_t* out_K,
                                      int8_t* out_labels, float* out_corr)
{
   if ( !ctx ) return KINC_SIM_EINVAL;
   int rc = check_range(ctx, start, size);
   if ( rc ) return rc;
   ctx->launches = 0;
   const int S = ctx->S;
   const int maxK = ctx->params.max_clusters * ctx->dp.ncorr;   /* floats per pair */
   for ( int64_t done = 0; done < size; )
   {
      const int64_t n = std::min<int64_t>(ctx->max_block, size - done);
      const int32_t before = ctx->launches;
      rc = enqueue_block(ctx, start + done, n, ctx->d_K, (out_labels && ctx->d_labels) ? ctx->d_labels : nullptr,
                         ctx->d_corr, ctx->stream);
      (void)before;
      if ( rc ) return rc;
      if ( out_K ) CK(cudaMemcpyAsync(out_K + done, ctx->d_K, n, cudaMemcpyDeviceToHost, ctx->stream));
      if ( out_labels && ctx->d_labels )
         CK(cudaMemcpyAsync(out_labels + done * S, ctx->d_labels, (size_t)n * S, cudaMemcpyDeviceToHost,
                            ctx->stream));
      if ( out_corr )
         CK(cudaMemcpyAsync(out_corr + done * maxK, ctx->d_corr, (size_t)n * maxK * sizeof(float),
                            cudaMemcpyDeviceToHost, ctx->stream));
      rc = kinc_sim_synchronize(ctx);
      if ( rc ) return rc;
      done += n;
   }
   return KINC_SIM_OK;
}

extern "C" int kinc_sim_execute_block_async(kinc_sim_ctx* ctx, int64_t start, int64_t size, int8_t* out_K,
                                            int8_t* out_labels, float* out_corr)
{
   if ( !ctx ) return KINC_SIM_EINVAL;
   int rc = check_range(ctx, start, size);
   if ( rc ) return rc;
   if ( size > ctx->max_block )
      return fail(ctx, KINC_SIM_EINVAL, "size %lld exceeds the device block limit %lld", (long long)size,
                  (long long)ctx->max_block);
   ctx->launches = 0;
   if ( size == 0 ) return KINC_SIM_OK;
   const int S = ctx->S;
   const int floats = ctx->params.max_clusters * ctx->dp.ncorr;   /* per pair */
   rc = enqueue_block(ctx, start, size, ctx->d_K, (out_labels && ctx->d_labels) ? ctx->d_labels : nullptr,
                      ctx->d_corr, ctx->stream);
   if ( rc ) return rc;
   if ( out_K ) CK(cudaMemcpyAsync(out_K, ctx->d_K, size, cudaMemcpyDeviceToHost, ctx->stream));
   if ( out_labels && ctx->d_labels )
      CK(cudaMemcpyAsync(out_labels, ctx->d_labels, (size_t)size * S, cudaMemcpyDeviceToHost, ctx->stream));
   if ( out_corr )
      CK(cudaMemcpyAsync(out_corr, ctx->d_corr, (size_t)size * floats * sizeof(float), cudaMemcpyDeviceToHost,
                         ctx->stream));
   return KINC_SIM_OK;
}

extern "C" int kinc_sim_compact_block_device(kinc_sim_ctx* ctx, int64_t start, int64_t size, const int8_t* d_K,
                                             const int8_t* d_labels, const float* d_corr, int32_t* cmx_x,
                                             int32_t* cmx_y, int8_t* cmx_c, float* cmx_r, int64_t cap_cmx,
                                             int32_t* ccm_x, int32_t* ccm_y, int8_t* ccm_c, uint8_t* ccm_packed,
                                             int64_t cap_ccm, uint64_t* d_counts, void* stream)
{
   if ( !ctx || !d_K || !d_corr || !d_counts ) return KINC_SIM_EINVAL;
   int rc = check_range(ctx, start, size);
   if ( rc ) return rc;
   if ( size > ctx->max_block )
      return fail(ctx, KINC_SIM_EINVAL, "size %lld exceeds the device block limit %lld", (long long)size,
                  (long long)ctx->max_block);
   if ( size == 0 ) return cudaMemsetAsync(d_counts, 0, 2 * sizeof(uint64_t),
                                           stream ? (cudaStream_t)stream : ctx->stream) == cudaSuccess
                             ? KINC_SIM_OK : KINC_SIM_ECUDA;
   cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
   CK(compact_enqueue(start, size, ctx->params.max_clusters, ctx->dp.ncorr, ctx->S, d_K, d_labels, d_corr,
                      ctx->params.min_corr,
                      ctx->params.max_corr, ctx->d_compact, cap_cmx, cap_ccm, cmx_x, cmx_y, cmx_c, cmx_r, ccm_x,
                      ccm_y, ccm_c, ccm_packed, (unsigned long long*)d_counts, st));
   return KINC_SIM_OK;
}

extern "C" int kinc_sim_pair_counts(kinc_sim_ctx* ctx, int64_t start, int64_t size, int32_t* out_N)
{
   if ( !ctx || !out_N ) return KINC_SIM_EINVAL;
   int rc = check_range(ctx, start, size);
   if ( rc ) return rc;
   for ( int64_t done = 0; done < size; )
   {
      const int64_t n = std::min<int64_t>(ctx->max_block, size - done);
      k_count<<<(int)std::min<int64_t>((n + 255) / 256, 65535), 256, 0, ctx->stream>>>(
         ctx->d_umask, ctx->W, start + done, n, ctx->d_N);
      CK(cudaGetLastError());
      CK(cudaMemcpyAsync(out_N + done, ctx->d_N, n * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
      CK(cudaStreamSynchronize(ctx->stream));
      done += n;
   }
   return KINC_SIM_OK;
}

extern "C" int kinc_sim_process_pairs(const kinc_sim_params* params, int32_t samples, int64_t start, int64_t size,
                                      const int8_t* K, const int8_t* labels, const float* corr, int32_t* cmx_x,
                                      int32_t* cmx_y, int8_t* cmx_c, float* cmx_r, int64_t cap_cmx,
                                      int64_t* n_cmx, int32_t* ccm_x, int32_t* ccm_y, int8_t* ccm_c,
                                      int8_t* ccm_codes, int64_t cap_ccm, int64_t* n_ccm)
{
   if ( !params || !K || !corr || samples < 1 || start < 0 || size < 0 )
      return fail(nullptr, KINC_SIM_EINVAL, "invalid arguments to kinc_sim_process_pairs");
   const int S = samples;
   const int maxK = params->max_clusters;
   const int ncorr = params->corr_method == 2 ? 2 : 1;   /* correlations per cluster */
   const float lo = params->min_corr;
   const float hi = params->max_corr;
   auto passes = [&](const float* r) {
      for ( int c = 0; c < ncorr; ++c )
         if ( !std::isnan(r[c]) && lo <= std::fabs(r[c]) && std::fabs(r[c]) <= hi ) return true;
      return false;
   };
   int64_t nc = 0, nm = 0;
   /* pair index -> (x, y) and then ++ (src/core/pairwise_index.cpp:32-57,85-94) */
   int64_t x = 1, pos = 0;
   while ( pos <= start ) { ++x; pos = x * (x - 1) / 2; }
   --x;
   int64_t y = start - x * (x - 1) / 2;
   for ( int64_t q = 0; q < size; ++q )
   {
      const int Kq = K[q];
      if ( Kq > 1 && labels && ccm_x )
      {
         int c = 0;
         for ( int k = 0; k < Kq; ++k )
         {
            if ( passes(corr + (q * maxK + k) * ncorr) )
            {
               if ( nm >= cap_ccm )
                  return fail(nullptr, KINC_SIM_EINVAL, "CCM capacity %lld exceeded", (long long)cap_ccm);
               ccm_x[nm] = (int32_t)x;
               ccm_y[nm] = (int32_t)y;
               ccm_c[nm] = (int8_t)c++;
               for ( int i = 0; i < S; ++i )
               {
                  const int8_t l = labels[q * S + i];
                  ccm_codes[nm * S + i] = (int8_t)(l >= 0 ? (k == l) : -l);
               }
               ++nm;
            }
         }
      }
      if ( Kq > 0 && cmx_x )
      {
         int c = 0;
         for ( int k = 0; k < Kq; ++k )
         {
            const float* r = corr + (q * maxK + k) * ncorr;
            if ( passes(r) )
            {
               if ( nc >= cap_cmx )
                  return fail(nullptr, KINC_SIM_EINVAL, "CMX capacity %lld exceeded", (long long)cap_cmx);
               cmx_x[nc] = (int32_t)x;
               cmx_y[nc] = (int32_t)y;
               cmx_c[nc] = (int8_t)c++;
               for ( int cc = 0; cc < ncorr; ++cc ) cmx_r[nc * ncorr + cc] = r[cc];
               ++nc;
            }
         }
      }
      if ( ++y >= x ) { y = 0; ++x; }
   }
   if ( n_cmx ) *n_cmx = nc;
   if ( n_ccm ) *n_ccm = nm;
   return KINC_SIM_OK;
}

extern "C" int kinc_sim_process_block(const kinc_sim_ctx* cctx, int64_t start, int64_t size, const int8_t* K,
                                      const int8_t* labels, const float* corr, int32_t* cmx_x, int32_t* cmx_y,
                                      int8_t* cmx_c, float* cmx_r, int64_t cap_cmx, int64_t* n_cmx,
                                      int32_t* ccm_x, int32_t* ccm_y, int8_t* ccm_c, int8_t* ccm_codes,
                                      int64_t cap_ccm, int64_t* n_ccm)
{
   kinc_sim_ctx* ctx = const_cast<kinc_sim_ctx*>(cctx);
   if ( !ctx ) return KINC_SIM_EINVAL;
   const int rc = kinc_sim_process_pairs(&ctx->params, ctx->S, start, size, K, labels, corr, cmx_x, cmx_y, cmx_c,
                                         cmx_r, cap_cmx, n_cmx, ccm_x, ccm_y, ccm_c, ccm_codes, cap_ccm, n_ccm);
   if ( rc ) ctx->err = g_create_error;
   return rc;
}

/* ======================================================= allocation-free
 *
 * kinc_sim_execute_block_noalloc: the same work as kinc_sim_execute_block_device
 * for callers that may not allocate device memory -- hosts that hand the
 * whole device to their own pool allocator and forbid raw cudaMalloc (which
 * also synchronises the device), or that run this step inside a region where
 * allocation is not allowed.  The caller passes its device expression matrix
 * and device outputs; everything else lives in the file-scope arrays below,
 * which every GPU that loads this library holds until the process exits.
 */
namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = (size_t)64 << 20;   /* 64 MiB of working memory */
constexpr int64_t NOALLOC_MAX_PAIRS = (int64_t)1 << 18;      /* pairs per call */
constexpr int NOALLOC_MAX_SAMPLES = 4096;
constexpr int NOALLOC_MAX_DEVICES = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];
static __device__ __align__(256) uint32_t g_noalloc_jump[RNG_BITS * RNG_WORDS * RNG_WORDS];
static __device__ __align__(256) uint32_t g_noalloc_rng0[RNG_WORDS];

struct NoallocDevice
{
   bool ready;
   unsigned char* scratch;     /* device address of g_noalloc_scratch on this device */
   uint32_t* jump;
   uint32_t* rng0;
};

NoallocDevice g_noalloc_dev[NOALLOC_MAX_DEVICES];
uint32_t g_noalloc_host_jump[RNG_BITS * RNG_WORDS * RNG_WORDS];
uint32_t g_noalloc_host_rng0[RNG_WORDS];
double g_noalloc_host_logn[NOALLOC_MAX_SAMPLES + 1];
bool g_noalloc_tables = false;
std::mutex g_noalloc_mutex;

/* the glibc rand() tables of glibc_rng_tables, computed into fixed storage */
void noalloc_rng_tables()
{
   int64_t r[344];
   r[0] = 1;
   for ( int i = 1; i < 31; ++i )
   {
      const int64_t hi = r[i - 1] / 127773;
      const int64_t lo = r[i - 1] % 127773;
      int64_t word = 16807 * lo - 2836 * hi;
      if ( word < 0 ) word += 2147483647;
      r[i] = word;
   }
   for ( int i = 31; i < 34; ++i ) r[i] = r[i - 31];
   for ( int i = 34; i < 344; ++i ) r[i] = (int64_t)(uint32_t)((uint32_t)r[i - 31] + (uint32_t)r[i - 3]);
   for ( int i = 0; i < RNG_WORDS; ++i ) g_noalloc_host_rng0[i] = (uint32_t)r[313 + i];
   const int n = RNG_WORDS;
   static uint32_t M[RNG_WORDS * RNG_WORDS], T[RNG_WORDS * RNG_WORDS];
   for ( int i = 0; i < n * n; ++i ) M[i] = 0u;
   for ( int i = 0; i < n - 1; ++i ) M[i * n + i + 1] = 1u;
   M[(n - 1) * n + 0] = 1u;
   M[(n - 1) * n + 28] = 1u;
   for ( int b = 0; b < RNG_BITS; ++b )
   {
      for ( int row = 0; row < n; ++row )
         for ( int c = 0; c < n; ++c ) g_noalloc_host_jump[(size_t)b * n * n + c * n + row] = M[row * n + c];
      for ( int i = 0; i < n; ++i )
         for ( int j = 0; j < n; ++j )
         {
            uint32_t acc = 0;
            for ( int k = 0; k < n; ++k ) acc += M[i * n + k] * M[k * n + j];
            T[i * n + j] = acc;
         }
      for ( int i = 0; i < n * n; ++i ) M[i] = T[i];
   }
}

/* the argument checks of validate(), with static messages (nothing allocated) */
const char* noalloc_check(const kinc_sim_params* p, int32_t G, int32_t S)
{
   if ( G < 2 ) return "genes must be >= 2";
   if ( S < 1 ) return "samples must be >= 1";
   if ( p->clus_method < 0 || p->clus_method > 2 ) return "clus_method must be 0 (none), 1 (gmm) or 2 (kmeans)";
   if ( p->corr_method < 0 || p->corr_method > 2 )
      return "corr_method must be 0 (pearson), 1 (spearman) or 2 (both)";
   if ( p->min_samples < 1 ) return "min_samples must be >= 1";
   if ( p->min_clusters < 1 || p->min_clusters > 64 ) return "min_clusters must be in 1..64";
   if ( p->max_clusters < 1 || p->max_clusters > 64 ) return "max_clusters must be in 1..64";
   if ( p->max_clusters < p->min_clusters ) return "Minimum clusters must be less than or equal to maximum clusters.";
   if ( p->criterion < 0 || p->criterion > 1 ) return "criterion must be 0 (BIC) or 1 (ICL)";
   if ( !(p->min_corr >= 0 && p->min_corr <= 1) || !(p->max_corr >= 0 && p->max_corr <= 1) )
      return "min_corr and max_corr must be in [0, 1]";
   if ( p->semantics < 0 || p->semantics > 1 ) return "semantics must be 0 or 1";
   if ( p->rand_mode < 0 || p->rand_mode > 1 ) return "rand_mode must be 0 or 1";
   if ( p->precision != 0 ) return "the allocation-free entry point runs the per-pair FP32 path only (precision 0)";
   return nullptr;
}

}  // namespace

extern "C" int kinc_sim_execute_block_noalloc(const float* d_gem, int32_t genes, int32_t samples,
                                              const kinc_sim_params* params, int64_t start, int64_t size,
                                              int8_t* d_K, int8_t* d_labels, float* d_corr, void* stream)
{
   kinc_sim_ctx* ctx = nullptr;   /* errors go to kinc_sim_last_error(NULL) of the calling thread */
   std::lock_guard<std::mutex> lock(g_noalloc_mutex);
   if ( !d_gem || !params ) return fail(nullptr, KINC_SIM_EINVAL, "d_gem and params must not be NULL");
   const char* bad = noalloc_check(params, genes, samples);
   if ( bad ) return fail(nullptr, KINC_SIM_EINVAL, "%s", bad);
   if ( samples > NOALLOC_MAX_SAMPLES )
      return fail(nullptr, KINC_SIM_EINVAL, "samples %d exceeds the allocation-free limit of %d", samples,
                  NOALLOC_MAX_SAMPLES);
   if ( size < 0 || size > NOALLOC_MAX_PAIRS )
      return fail(nullptr, KINC_SIM_EINVAL, "size %lld exceeds the allocation-free limit of %lld pairs per call",
                  (long long)size, (long long)NOALLOC_MAX_PAIRS);
   const int64_t total = (int64_t)genes * (genes - 1) / 2;
   if ( start < 0 || start + size > total )
      return fail(nullptr, KINC_SIM_EINVAL, "pair range [%lld, %lld) outside [0, %lld)", (long long)start,
                  (long long)(start + size), (long long)total);
   if ( size == 0 ) return KINC_SIM_OK;

   int dev = 0;
   CK(cudaGetDevice(&dev));
   if ( dev < 0 || dev >= NOALLOC_MAX_DEVICES )
      return fail(nullptr, KINC_SIM_EINVAL, "device %d beyond the supported %d", dev, NOALLOC_MAX_DEVICES);
   cudaStream_t st = (cudaStream_t)stream;

   /* set-up, once per device, with that device current */
   NoallocDevice& nd = g_noalloc_dev[dev];
   if ( !nd.ready )
   {
      void* p = nullptr;
      CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
      nd.scratch = (unsigned char*)p;
      CK(cudaGetSymbolAddress(&p, g_noalloc_jump));
      nd.jump = (uint32_t*)p;
      CK(cudaGetSymbolAddress(&p, g_noalloc_rng0));
      nd.rng0 = (uint32_t*)p;
      if ( !g_noalloc_tables )
      {
         noalloc_rng_tables();
         g_noalloc_tables = true;
      }
      CK(cudaMemcpyToSymbol(g_noalloc_jump, g_noalloc_host_jump, sizeof g_noalloc_host_jump));
      CK(cudaMemcpyToSymbol(g_noalloc_rng0, g_noalloc_host_rng0, sizeof g_noalloc_host_rng0));
      nd.ready = true;
   }

   /* device parameters, as kinc_sim_create derives them */
   const int S = samples;
   const int W = (S + 31) / 32;
   DevParams dp {};
   dp.G = genes; dp.S = S; dp.W = W;
   dp.clus = params->clus_method; dp.corr = params->corr_method;
   dp.min_expr = params->min_expr; dp.min_samples = params->min_samples;
   dp.min_k = params->min_clusters; dp.max_k = params->max_clusters;
   dp.criterion = params->criterion; dp.pre_out = params->pre_out; dp.post_out = params->post_out;
   dp.semantics = params->semantics; dp.rand_mode = params->rand_mode;
   dp.draws_per_pair = draws_per_pair(*params);
   dp.c2 = 2 * std::log(2.0f * M_PI);
   dp.neg_zero = -0.0f;
   dp.P2 = next_pow2_host(std::max(S, 2));
   const bool need_sort = (params->clus_method != 0 && (params->pre_out || params->post_out))
                          || params->corr_method >= 1;
   dp.sort_floats = params->corr_method >= 1 ? 3 * dp.P2 : (need_sort ? dp.P2 : 0);
   /* room for the GMM responsibilities the fit keeps between its two M passes (as in kinc_sim_create) */
   dp.gam_k = (KINC_STORE_GAMMA && params->clus_method == 1)
                 ? (params->max_clusters <= 3 ? 3 : params->max_clusters <= 5 ? 5 : 0) : 0;
   dp.ncorr = params->corr_method == 2 ? 2 : 1;
   const size_t sort_bytes_warp = (size_t)dp.sort_floats * sizeof(float);
   const SimKernel kern = params->clus_method == 0 ? sim_kernel_none()
                        : params->clus_method == 1 ? sim_kernel_gmm(params->max_clusters, params->rand_mode == 1)
                                                   : sim_kernel_kmeans(params->max_clusters);
   const int wpb = kern.wpb;
   {
      const kinc_sim_launch l = default_launch(kern, params->clus_method);
      dp.warps = l.warps_per_cta;
      dp.rounds = l.rounds;
      dp.prefetch = l.prefetch;
   }
   const size_t param_bytes_warp = (KINC_GMM_PARAMS_SMEM && kern.clus == 1 && kern.ks > 0)
                                      ? (size_t)7 * kern.ks * TILE * sizeof(float) : 0;
   const KmPool km = km_pool_sizes(*params, kern);
   dp.km_dmax = km.dmax;
   dp.km_tmax = km.tmax;
   const int smem_sort = need_sort && param_bytes_warp == 0 && sort_bytes_warp * wpb <= 200 * 1024;
   const int smem_bytes = (int)((smem_sort ? sort_bytes_warp : 0) + param_bytes_warp) * wpb;
   if ( smem_bytes > 0 )
      CK(cudaFuncSetAttribute(kern.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes));

   /* carve the static array: fixed parts first, then as many warp slots as fit */
   size_t off = 0;
   auto take = [&](size_t bytes) {
      const size_t o = off;
      off += (bytes + 255) & ~(size_t)255;
      return o;
   };
   const int64_t lo = (start / KINC_SIM_WORK_BLOCK_SIZE) * KINC_SIM_WORK_BLOCK_SIZE;
   const int64_t end = start + size;
   const int64_t span = end - lo;
   const int nscan = (int)((size + SCAN_THREADS - 1) / SCAN_THREADS);
   const size_t oMask = take((size_t)genes * W * sizeof(uint32_t));
   const size_t oLogn = take((size_t)(S + 1) * sizeof(double));
   const size_t oN = take((size_t)span * sizeof(int32_t));
   const size_t oPg = take((size_t)span * sizeof(int32_t));
   const size_t oQ = take((size_t)size * sizeof(uint64_t));
   const size_t oBsum = take((size_t)(nscan + 1) * sizeof(unsigned long long));
   const size_t oSmall = take(8 * sizeof(unsigned long long));
   const size_t col = (size_t)S * TILE;
   const size_t slot_bytes = ((col * sizeof(float2) + 255) & ~(size_t)255) + ((col * sizeof(float) + 255) & ~(size_t)255)
                             + ((col * sizeof(float) * dp.gam_k + 255) & ~(size_t)255)
                             + 5 * ((col + 255) & ~(size_t)255)
                             + (((size_t)RNG_WORDS * TILE * sizeof(uint32_t) + 255) & ~(size_t)255)
                             + (smem_sort ? 0 : ((sort_bytes_warp + 255) & ~(size_t)255))
                             + ((params->clus_method == 2 && KINC_KMEANS_LANE_MAJOR && kern.ks == 0)
                                   ? ((col * sizeof(float2) + 255) & ~(size_t)255) : 0)
                             + km.bytes;
   if ( off >= NOALLOC_SCRATCH_BYTES || (NOALLOC_SCRATCH_BYTES - off) / slot_bytes < (size_t)wpb )
      return fail(nullptr, KINC_SIM_EINVAL,
                  "%d genes x %d samples and %lld pairs do not fit the %zu-byte allocation-free scratch",
                  genes, samples, (long long)size, NOALLOC_SCRATCH_BYTES);
   const size_t nslots = ((NOALLOC_SCRATCH_BYTES - off) / slot_bytes) / wpb * wpb;
   unsigned char* base = nd.scratch;
   DevScratch ds {};
   {
      size_t o = off;
      auto carve = [&](size_t bytes) {
         unsigned char* p = base + o;
         o += (bytes + 255) & ~(size_t)255;
         return p;
      };
      ds.X = (float2*)carve(nslots * col * sizeof(float2));
      ds.lpx = (float*)carve(nslots * col * sizeof(float));
      ds.gam = dp.gam_k ? (float*)carve(nslots * col * sizeof(float) * dp.gam_k) : nullptr;
      ds.lbl = (int8_t*)carve(nslots * col);
      ds.wl = (int8_t*)carve(nslots * col);
      ds.ya = (int8_t*)carve(nslots * col);
      ds.yb = (int8_t*)carve(nslots * col);
      ds.yc = (int8_t*)carve(nslots * col);
      ds.rng = (uint32_t*)carve(nslots * RNG_WORDS * TILE * sizeof(uint32_t));
      ds.sortbuf = smem_sort ? nullptr : (float*)carve(nslots * sort_bytes_warp);
      ds.Xl = (params->clus_method == 2 && KINC_KMEANS_LANE_MAJOR && kern.ks == 0)
                 ? (float2*)carve(nslots * col * sizeof(float2)) : nullptr;
      ds.kmd = km.bytes ? (int32_t*)carve(nslots * (size_t)km.dmax * TILE * sizeof(int32_t)) : nullptr;
      ds.kmr = km.bytes ? (float*)carve(nslots * (size_t)km.tmax * km.rs * sizeof(float)) : nullptr;
      if ( o > NOALLOC_SCRATCH_BYTES )
         return fail(nullptr, KINC_SIM_EINVAL, "allocation-free scratch layout overflow");
   }
   uint32_t* d_umask = (uint32_t*)(base + oMask);
   double* d_logn = (double*)(base + oLogn);
   int32_t* d_N = (int32_t*)(base + oN);
   int32_t* d_pg = (int32_t*)(base + oPg);
   uint64_t* d_qpos = (uint64_t*)(base + oQ);
   unsigned long long* d_bsum = (unsigned long long*)(base + oBsum);
   unsigned long long* small = (unsigned long long*)(base + oSmall);
   unsigned long long* d_qbase = small + 0;
   unsigned long long* d_tiles = small + 1;
   unsigned long long* d_work = small + 2;      /* 4 words */
   int* d_status = (int*)(small + 6);

   /* every call shares the array: clear what must start at zero */
   CK(cudaMemsetAsync(small, 0, 8 * sizeof(unsigned long long), st));
   for ( int n = 0; n <= S; ++n ) g_noalloc_host_logn[n] = std::log((double)n);
   CK(cudaMemcpyAsync(d_logn, g_noalloc_host_logn, (size_t)(S + 1) * sizeof(double), cudaMemcpyHostToDevice, st));
   k_masks<<<std::max(1, std::min(65535, (int)(((int64_t)genes * W + 255) / 256))), 256, 0, st>>>(
      d_gem, genes, S, W, params->min_expr, d_umask);
   k_count<<<(int)std::min<int64_t>((span + 255) / 256, 65535), 256, 0, st>>>(d_umask, W, lo, span, d_N);
   if ( dp.clus != 0 && dp.rand_mode == 0 )
   {
      if ( start > 0 )
         k_count_qualifying<<<1024, 256, 0, st>>>(d_umask, W, start, dp.min_samples, d_qbase);
      const int64_t offq = start - lo;
      k_scan_sums<<<nscan, SCAN_THREADS, 0, st>>>(d_N, offq, size, dp.min_samples, d_bsum);
      k_scan_blocks<<<1, SCAN_THREADS, 0, st>>>(d_bsum, nscan, d_qbase);
      k_scan_apply<<<nscan, SCAN_THREADS, 0, st>>>(d_N, offq, size, dp.min_samples, d_bsum, d_qpos);
   }
   if ( (dp.corr == 0 || dp.corr == 2) && dp.semantics == 0 )
   {
      CK(launch_prev(d_N, lo, end, d_pg, st));
   }
   CK(cudaGetLastError());
   DevData dd {};
   dd.gem = d_gem;
   dd.umask = d_umask;
   dd.logn = d_logn;
   dd.jump = nd.jump;
   dd.rng0 = nd.rng0;
   DevBlock B {};
   B.start = start;
   B.size = size;
   B.lo = lo;
   B.N = d_N;
   B.pg = d_pg;
   B.qpos = d_qpos;
   B.order = nullptr;
   B.outK = d_K;
   B.outLabels = d_labels;
   B.outCorr = d_corr;
   B.tiles = d_tiles;
   B.status = d_status;
   B.work = d_work;
   const int grid = (int)(nslots / wpb);
   cudaError_t e = kern.clus == 0 ? sim_launch_none(kern, grid, smem_bytes, st, dp, dd, ds, B, smem_sort)
                 : kern.clus == 1 ? sim_launch_gmm(kern, grid, smem_bytes, st, dp, dd, ds, B, smem_sort)
                                  : sim_launch_kmeans(kern, grid, smem_bytes, st, dp, dd, ds, B, smem_sort);
   CK(e);

   /* the scratch is shared by every call: finish before the next one reuses it */
   CK(cudaStreamSynchronize(st));
   int status = 0;
   CK(cudaMemcpy(&status, d_status, sizeof(int), cudaMemcpyDeviceToHost));
   if ( status != ST_OK ) return fail(nullptr, KINC_SIM_EKERNEL, "kernel reported status %d", status);
   return KINC_SIM_OK;
}
