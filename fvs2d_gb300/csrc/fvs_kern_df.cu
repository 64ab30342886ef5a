// fvs_kern_df.cu — device kernels, FP64 accuracy on the FP32 pipe: gradient,
// limiter, reconstruction, Roe flux, the slot gather and the RK stage in
// double-float (df64, 48-bit significand); the state stored in FP64, FP64
// local time step, norms summed as FP32 pairs.
#define FVS_NS k_df
#define FVS_T df64
#define FVS_MIXED 0
#define FVS_STRICT 0
#define FVS_DF 1
#include "fvs_kernels.cuh"

namespace fvs {
const KernelSet& kernels_fp64_df() {
  static const KernelSet k = {"fp64_df", k_df::launch_begin_step, k_df::launch_cvar2pvar, k_df::launch_gradient,
                              k_df::launch_flux, k_df::launch_update, k_df::launch_residual_out, k_df::persistent_occupancy, k_df::launch_persistent, k_df::launch_tiled_step,
                              k_df::launch_tile_stage, k_df::tile_smem,
                              k_df::launch_tile_fu_stage, nullptr, nullptr, nullptr,
                              k_df::update_wave};
  return k;
}
}  // namespace fvs
