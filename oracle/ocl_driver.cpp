/*
 * TEST INFRASTRUCTURE ONLY.  Appended by oracle/build_ref.py to KINC's OpenCL kernels
 * compiled as C++ (ref_shim/ocl_shim.h), it runs them the way KINC's OpenCL worker does, on
 * the CPU, one work item after another.
 *
 * Restated here (the originals need ACE and an OpenCL runtime):
 *   Similarity::OpenCL::Worker::Worker   src/core/similarity_opencl_worker.cpp:50-86 (slot buffers)
 *   Similarity::OpenCL::Worker::execute  src/core/similarity_opencl_worker.cpp:93-271
 *   the kernel-argument wrappers         src/core/similarity_opencl_{fetchpair,gmm,pearson,spearman}.cpp
 *   Pairwise::Index(qint64), ++          src/core/pairwise_index.cpp:32-57,85-94
 * One worker serves the whole call, as one ACE worker serves consecutive work blocks: its slot
 * buffers keep their contents from chunk to chunk and block to block.  OpenCL leaves a new
 * buffer's contents undefined; they are zeros here.  Each work block of 32,768 pairs is cut into
 * chunks of ksize work items, the last one padded with index (0, 0).  The host passes minexpr
 * to the fetchPair kernel as an int (src/core/similarity_opencl_fetchpair.h:28), converted here
 * with saturation (-inf gives INT_MIN, as x86 and Arm convert it).
 * K-means is not driven: its kernel indexes past the work buffers the worker allocates
 * (src/opencl/kmeans.cl:104-113 against src/core/similarity_opencl_worker.cpp:72).
 */
#include <algorithm>
#include <climits>
#include <cstring>
#include <vector>

thread_local int kocl_global_id = 0;

namespace {

constexpr int64_t WORK_BLOCK = 32768;

void kocl_decode(int64_t index, int& x, int& y)
{
   int64_t xx = 1, pos = 0;
   while ( pos + xx <= index )
   {
      pos += xx;
      ++xx;
   }
   x = (int)xx;
   y = (int)(index - pos);
}

int kocl_int_of(float v)
{
   if ( std::isnan(v) ) return 0;
   if ( v <= (float)INT_MIN ) return INT_MIN;
   if ( v >= (float)INT_MAX ) return INT_MAX;
   return (int)v;
}

}  // namespace

extern "C" {

typedef struct kocl_params
{
   int clus_method;   /* 0 none, 1 GMM (K-means is not driven) */
   int corr_method;   /* 0 Pearson, 1 Spearman */
   float min_expr;
   int min_samples;
   int min_clusters;
   int max_clusters;
   int criterion;     /* 0 BIC, 1 ICL */
   int pre_out;
   int post_out;
   int ksize;
} kocl_params;

/* Pairs [start, start + size): K int8[size], labels int8[size][S] (rows with K > 1),
 * corr float[size][max_clusters] (rows with K > 0, all max_clusters values as the worker
 * returns them).  Returns 0, or -1 for arguments the worker would not run. */
int kocl_run(const float* gem, int G, int S, const kocl_params* p, int64_t start, int64_t size, int8_t* outK,
             int8_t* outLabels, float* outCorr)
{
   if ( !gem || !p || G < 2 || S < 1 || size < 0 || start < 0 || p->ksize < 1 || p->max_clusters < 1
        || p->max_clusters > 64 || p->clus_method < 0 || p->clus_method > 1 || p->corr_method < 0
        || p->corr_method > 1 || start + size > (int64_t)G * (G - 1) / 2 )
      return -1;
   const int ks = p->ksize, K = p->max_clusters, Np2 = nextPower2(S);
   /* the worker's slot buffers */
   std::vector<int2> in_index((size_t)ks);
   std::vector<Vector2> work_X((size_t)S * ks);
   std::vector<int> work_N((size_t)ks);
   std::vector<char> work_labels((size_t)S * ks);
   std::vector<Component> work_components((size_t)K * ks);
   std::vector<Vector2> work_MP((size_t)K * ks);
   std::vector<int> work_counts((size_t)K * ks);
   std::vector<float> work_logpi((size_t)K * ks), work_loggamma((size_t)S * K * ks), work_logGamma((size_t)K * ks);
   std::vector<char> out_K((size_t)ks), out_labels((size_t)S * ks);
   std::vector<float> work_x((size_t)Np2 * ks), work_y((size_t)Np2 * ks), out_corr((size_t)K * ks);
   std::vector<int> work_rank((size_t)Np2 * ks);
   memset((void*)work_X.data(), 0, work_X.size() * sizeof(Vector2));
   memset((void*)work_components.data(), 0, work_components.size() * sizeof(Component));
   memset((void*)work_MP.data(), 0, work_MP.size() * sizeof(Vector2));
   const int minexpr = kocl_int_of(p->min_expr);

   int64_t done = 0;
   while ( done < size )
   {
      /* one work block: from the pair at `done` to the next multiple of 32,768 */
      const int64_t b0 = start + done;
      const int64_t b1 = std::min(start + size, (b0 / WORK_BLOCK + 1) * WORK_BLOCK);
      int x = 0, y = 0;
      kocl_decode(b0, x, y);
      for ( int64_t c0 = b0; c0 < b1; c0 += ks )
      {
         const int steps = (int)std::min<int64_t>(ks, b1 - c0);
         for ( int j = 0; j < steps; ++j )
         {
            in_index[(size_t)j] = { x, y };
            if ( ++y >= x )
            {
               ++x;
               y = 0;
            }
         }
         for ( int j = steps; j < ks; ++j ) in_index[(size_t)j] = { 0, 0 };

         for ( int j = 0; j < ks; ++j )
         {
            kocl_global_id = j;
            fetchPair(gem, S, in_index.data(), minexpr, work_X.data(), work_N.data(), out_labels.data());
         }
         if ( p->clus_method == 1 )
         {
            for ( int j = 0; j < ks; ++j )
            {
               kocl_global_id = j;
               GMM_compute(gem, S, p->min_samples, (char)p->min_clusters, (char)p->max_clusters,
                           (Criterion)p->criterion, p->pre_out, p->post_out, work_X.data(), work_N.data(),
                           work_labels.data(), work_components.data(), work_MP.data(), work_counts.data(),
                           work_logpi.data(), work_loggamma.data(), work_logGamma.data(), out_K.data(),
                           out_labels.data());
            }
         }
         else
         {
            for ( int j = 0; j < ks; ++j ) out_K[(size_t)j] = 1;
         }
         const float2* data = reinterpret_cast<const float2*>(work_X.data());
         for ( int j = 0; j < ks; ++j )
         {
            kocl_global_id = j;
            if ( p->corr_method == 0 )
               Pearson_compute(data, (char)K, out_labels.data(), S, p->min_samples, out_corr.data());
            else
               Spearman_compute(data, (char)K, out_labels.data(), S, p->min_samples, work_x.data(), work_y.data(),
                                work_rank.data(), out_corr.data());
         }
         for ( int j = 0; j < steps; ++j )
         {
            const int64_t o = c0 - start + j;
            outK[o] = (int8_t)out_K[(size_t)j];
            memcpy(outLabels + o * S, out_labels.data() + (size_t)j * S, (size_t)S);
            memcpy(outCorr + o * K, out_corr.data() + (size_t)j * K, sizeof(float) * (size_t)K);
         }
      }
      done = b1 - start;
   }
   return 0;
}

}  // extern "C"
