// fvs_kern_mixed.cu — device kernels, mixed precision: FP32 gradient, limiter, reconstruction and Roe flux;
// residual sums exact (TwoSum), the RK increment in FP32 added to the FP64 state, FP64 local time step, norms
// summed as FP32 pairs.
#define FVS_NS k_mixed
#define FVS_T float
#define FVS_MIXED 1
#define FVS_STRICT 0
#include "fvs_kernels.cuh"

namespace fvs {
const KernelSet& kernels_mixed() {
  static const KernelSet k = {"mixed", k_mixed::launch_begin_step, k_mixed::launch_cvar2pvar, k_mixed::launch_gradient,
                              k_mixed::launch_flux, k_mixed::launch_update, k_mixed::launch_residual_out, k_mixed::persistent_occupancy,
                              k_mixed::launch_persistent, k_mixed::launch_tiled_step,
                              k_mixed::launch_tile_stage, k_mixed::tile_smem,
                              k_mixed::launch_tile_fu_stage, k_mixed::launch_tile_dma_stage,
                              k_mixed::tile_dma_smem, k_mixed::launch_tile_dma_fill,
                              k_mixed::update_wave};
  return k;
}
const DcKernels& dc_kernels() {
  static const DcKernels k = {k_mixed::dc_fold, k_mixed::dc_base, k_mixed::dc_occupancy, k_mixed::dc_persistent,
                              k_mixed::dc_tiled_step};
  return k;
}
}  // namespace fvs
