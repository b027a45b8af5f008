// pimc_fused.cu -- the fused sweep kernels (every phase of a sweep in one
// launch; one CTA or one warp per chain), in a translation unit of their own
// so that they compile in parallel with the rest.
#include <cuda_runtime.h>

#include "pimc_sweep.cuh"

namespace pimc {

// one CTA per chain, every phase of the sweep in one launch
__global__ void __launch_bounds__(512, 1) k_sweep(SweepArgs a) { sweep_cta<SW_ALL>(a); }
// one warp per chain, every phase
__global__ void __launch_bounds__(256, 2) k_sweep_warp(SweepArgs a) { sweep_warp<SW_ALL>(a); }

cudaError_t launch_sweep(const SweepArgs &a, int mode, int grid, int block, size_t smem,
                         cudaStream_t s) {
  if (mode == 1) k_sweep_warp<<<grid, block, smem, s>>>(a);
  else k_sweep<<<grid, block, smem, s>>>(a);
  return cudaGetLastError();
}
cudaError_t sweep_set_smem(int mode, size_t smem) {
  if (mode == 1)
    return cudaFuncSetAttribute(k_sweep_warp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  return cudaFuncSetAttribute(k_sweep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}
cudaError_t sweep_occupancy(int mode, int block, size_t smem, int *blocks_per_sm) {
  if (mode == 1)
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_sweep_warp, block, smem);
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_sweep, block, smem);
}
PIMC_UNIT_ACCESSORS(fused)

}  // namespace pimc
