// Instantiations of the fused stage kernel for orders 14 15 (one translation
// unit per group so that the build compiles them in parallel).
#include "sdg_stage_order.cuh"

namespace sdg {
int launch_stage_p14(int prec, int opt, const StageArgs& a, cudaStream_t st) {
  return launch_stage_order<14>(prec, opt, a, st);
}
int launch_stage_p15(int prec, int opt, const StageArgs& a, cudaStream_t st) {
  return launch_stage_order<15>(prec, opt, a, st);
}
}  // namespace sdg
