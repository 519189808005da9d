// Instantiations of the fused stage kernel for orders 12 13 (one translation
// unit per group so that the build compiles them in parallel).
#include "sdg_stage_order.cuh"

namespace sdg {
int launch_stage_p12(int prec, int opt, const StageArgs& a, cudaStream_t st) {
  return launch_stage_order<12>(prec, opt, a, st);
}
int launch_stage_p13(int prec, int opt, const StageArgs& a, cudaStream_t st) {
  return launch_stage_order<13>(prec, opt, a, st);
}
}  // namespace sdg
