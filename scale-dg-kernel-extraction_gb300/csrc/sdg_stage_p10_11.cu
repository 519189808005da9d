// Instantiations of the fused stage kernel for orders 10 11 (one translation
// unit per group so that the build compiles them in parallel).
#include "sdg_stage_order.cuh"

namespace sdg {
int launch_stage_p10(int prec, int opt, const StageArgs& a, cudaStream_t st) {
  return launch_stage_order<10>(prec, opt, a, st);
}
int launch_stage_p11(int prec, int opt, const StageArgs& a, cudaStream_t st) {
  return launch_stage_order<11>(prec, opt, a, st);
}
}  // namespace sdg
