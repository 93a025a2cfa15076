/* Similarity kernel specialisations with K-means clustering: register-resident
 * centroids up to K = 3 or 5, local-memory centroids beyond. */
#include "sim_kernel.cuh"

namespace kinc {

SimKernel sim_kernel_kmeans(int max_k)
{
   if ( max_k <= 3 ) return sim_kernel_handle<2, 3>();
   if ( max_k <= 5 ) return sim_kernel_handle<2, 5>();
   return sim_kernel_handle<2, 0>();
}

cudaError_t sim_launch_kmeans(const SimKernel& k, int grid, int smem, cudaStream_t st, const DevParams& P,
                              const DevData& D, const DevScratch& W, const DevBlock& B, int smem_sort)
{
   switch ( k.ks )
   {
   case 3: return sim_kernel_launch<2, 3>(grid, smem, st, P, D, W, B, smem_sort);
   case 5: return sim_kernel_launch<2, 5>(grid, smem, st, P, D, W, B, smem_sort);
   default: return sim_kernel_launch<2, 0>(grid, smem, st, P, D, W, B, smem_sort);
   }
}

} /* namespace kinc */
