/* Similarity kernel specialisations with GMM clustering: register-resident
 * components up to K = 3 or 5, local-memory components beyond; each in the
 * CPU path's form (CLUS 1) and the OpenCL kernels' form (CLUS 3, rand_mode 1). */
#include "sim_kernel.cuh"

namespace kinc {

SimKernel sim_kernel_gmm(int max_k, bool opencl)
{
   if ( opencl )
   {
      if ( max_k <= 3 ) return sim_kernel_handle<3, 3>();
      if ( max_k <= 5 ) return sim_kernel_handle<3, 5>();
      return sim_kernel_handle<3, 0>();
   }
   if ( max_k <= 3 ) return sim_kernel_handle<1, 3>();
   if ( max_k <= 5 ) return sim_kernel_handle<1, 5>();
   return sim_kernel_handle<1, 0>();
}

cudaError_t sim_launch_gmm(const SimKernel& k, int grid, int smem, cudaStream_t st, const DevParams& P,
                           const DevData& D, const DevScratch& W, const DevBlock& B, int smem_sort)
{
   if ( k.ocl )
   {
      switch ( k.ks )
      {
      case 3: return sim_kernel_launch<3, 3>(grid, smem, st, P, D, W, B, smem_sort);
      case 5: return sim_kernel_launch<3, 5>(grid, smem, st, P, D, W, B, smem_sort);
      default: return sim_kernel_launch<3, 0>(grid, smem, st, P, D, W, B, smem_sort);
      }
   }
   switch ( k.ks )
   {
   case 3: return sim_kernel_launch<1, 3>(grid, smem, st, P, D, W, B, smem_sort);
   case 5: return sim_kernel_launch<1, 5>(grid, smem, st, P, D, W, B, smem_sort);
   default: return sim_kernel_launch<1, 0>(grid, smem, st, P, D, W, B, smem_sort);
   }
}

} /* namespace kinc */
