// pimc_swap.cu -- the swap-phase kernels of the split sweep, in a
// translation unit of their own so that they compile in parallel with the
// rest (pimc_sweep.cu); the host reaches them through the launchers below.
#include <cuda_runtime.h>

#include "pimc_sweep.cuh"

namespace pimc {

// one CTA per chain (the generic swap)
__global__ void __launch_bounds__(512, 1) k_sweep_swap(SweepArgs a) { sweep_cta<SW_SWAP>(a); }
// the swap launch for batches whose every chain follows the reference's
// rules without a hard core or a contact table (swap_group SWAP_REF)
__global__ void __launch_bounds__(512, 1) k_sweep_swap_ref(SweepArgs a) {
  sweep_cta<SW_SWAP, SWAP_REF>(a);
}
// both for CTAs of at most 64 threads, compiled for 6 and 4 resident CTAs
// per SM: up to 170 and 255 registers a thread instead of 128 (fewer
// spills, fewer chains in flight)
__global__ void __launch_bounds__(64, 6) k_sweep_swap_r170(SweepArgs a) { sweep_cta<SW_SWAP>(a); }
__global__ void __launch_bounds__(64, 4) k_sweep_swap_r255(SweepArgs a) { sweep_cta<SW_SWAP>(a); }
__global__ void __launch_bounds__(64, 6) k_sweep_swap_ref_r170(SweepArgs a) {
  sweep_cta<SW_SWAP, SWAP_REF>(a);
}
__global__ void __launch_bounds__(64, 4) k_sweep_swap_ref_r255(SweepArgs a) {
  sweep_cta<SW_SWAP, SWAP_REF>(a);
}
// one warp per chain: twice the chains in flight of a two-warp CTA per chain
// at the same registers per SM
__global__ void __launch_bounds__(256, 2) k_sweep_swap_warp(SweepArgs a) { sweep_warp<SW_SWAP>(a); }

// regs: 0 (the 128-register kernels), 170 or 255
const void *swap_kernel(int warp, int spec, int regs) {
  if (warp) return (const void *)k_sweep_swap_warp;
  if (regs == 170) return spec ? (const void *)k_sweep_swap_ref_r170 : (const void *)k_sweep_swap_r170;
  if (regs == 255) return spec ? (const void *)k_sweep_swap_ref_r255 : (const void *)k_sweep_swap_r255;
  return spec ? (const void *)k_sweep_swap_ref : (const void *)k_sweep_swap;
}

cudaError_t launch_swap(const SweepArgs &a, int warp, int spec, int regs, int grid, int block,
                        size_t smem, cudaStream_t s) {
  if (warp) k_sweep_swap_warp<<<grid, block, smem, s>>>(a);
  else if (regs == 170 && spec) k_sweep_swap_ref_r170<<<grid, block, smem, s>>>(a);
  else if (regs == 170) k_sweep_swap_r170<<<grid, block, smem, s>>>(a);
  else if (regs == 255 && spec) k_sweep_swap_ref_r255<<<grid, block, smem, s>>>(a);
  else if (regs == 255) k_sweep_swap_r255<<<grid, block, smem, s>>>(a);
  else if (spec) k_sweep_swap_ref<<<grid, block, smem, s>>>(a);
  else k_sweep_swap<<<grid, block, smem, s>>>(a);
  return cudaGetLastError();
}

PIMC_UNIT_ACCESSORS(swap)

}  // namespace pimc
