// fvs_kern_strict.cu — device kernels, FP64, compiled with -fmad=false: no multiply-add contraction, so every
// rounding matches the CPU oracle built with -ffp-contract=off.
#define FVS_NS k_strict
#define FVS_T double
#define FVS_MIXED 0
#define FVS_STRICT 1
#include "fvs_kernels.cuh"

namespace fvs {
const KernelSet& kernels_fp64_strict() {
  static const KernelSet k = {"strict", k_strict::launch_begin_step, k_strict::launch_cvar2pvar, k_strict::launch_gradient,
                              k_strict::launch_flux, k_strict::launch_update, k_strict::launch_residual_out, k_strict::persistent_occupancy,
                              k_strict::launch_persistent, k_strict::launch_tiled_step,
                              nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                              k_strict::update_wave};
  return k;
}
}  // namespace fvs
