// fvs_kern_bounds.cu — device kernels, FP64 with multiply-add contraction (the
// FVS_PREC_FP64 arithmetic) and every indirect index checked (FVS_BOUNDS):
// the index-checking build that FVS2D_BOUNDS=1 handles run.
#define FVS_NS k_bounds
#define FVS_T double
#define FVS_MIXED 0
#define FVS_STRICT 0
#define FVS_BOUNDS 1
#include "fvs_kernels.cuh"

namespace fvs {
const KernelSet& kernels_fp64_bounds() {
  static const KernelSet k = {"fp64_bounds", k_bounds::launch_begin_step, k_bounds::launch_cvar2pvar,
                              k_bounds::launch_gradient, k_bounds::launch_flux, k_bounds::launch_update,
                              k_bounds::launch_residual_out, k_bounds::persistent_occupancy,
                              k_bounds::launch_persistent, k_bounds::launch_tiled_step, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                              k_bounds::update_wave};
  return k;
}
}  // namespace fvs
