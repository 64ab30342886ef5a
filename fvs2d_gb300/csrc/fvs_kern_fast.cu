// fvs_kern_fast.cu — device kernels, FP64, compiled with -fmad=true (multiply-add contraction allowed).
#define FVS_NS k_fast
#define FVS_T double
#define FVS_MIXED 0
#define FVS_STRICT 0
#include "fvs_kernels.cuh"

namespace fvs {
const KernelSet& kernels_fp64_fast() {
  static const KernelSet k = {"fast", k_fast::launch_begin_step, k_fast::launch_cvar2pvar, k_fast::launch_gradient,
                              k_fast::launch_flux, k_fast::launch_update, k_fast::launch_residual_out, k_fast::persistent_occupancy,
                              k_fast::launch_persistent, k_fast::launch_tiled_step,
                              nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                              k_fast::update_wave};
  return k;
}
}  // namespace fvs
