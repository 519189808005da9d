// Instantiations of the fused stage kernel for orders 5 6 (one translation
// unit per group so that the build compiles them in parallel).
#include "sdg_stage_order.cuh"

namespace sdg {
int launch_stage_p5(int prec, int opt, const StageArgs& a, cudaStream_t st) {
  return launch_stage_order<5>(prec, opt, a, st);
}
int launch_stage_p6(int prec, int opt, const StageArgs& a, cudaStream_t st) {
  return launch_stage_order<6>(prec, opt, a, st);
}
}  // namespace sdg
