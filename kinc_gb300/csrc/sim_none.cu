/* Similarity kernel specialisation without clustering (clusmethod none). */
#include "sim_kernel.cuh"

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

} /* namespace kinc */
