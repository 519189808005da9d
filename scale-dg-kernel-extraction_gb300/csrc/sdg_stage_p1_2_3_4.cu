// Instantiations of the fused stage kernel for orders 1 2 3 4 (one translation
// unit per group so that the build compiles them in parallel).
#include "sdg_stage_order.cuh"

namespace sdg {
int launch_stage_p1(int prec, int opt, const StageArgs& a, cudaStream_t st) {
  return launch_stage_order<1>(prec, opt, a, st);
}
int launch_stage_p2(int prec, int opt, const StageArgs& a, cudaStream_t st) {
  return launch_stage_order<2>(prec, opt, a, st);
}
int launch_stage_p3(int prec, int opt, const StageArgs& a, cudaStream_t st) {
  return launch_stage_order<3>(prec, opt, a, st);
}
int launch_stage_p4(int prec, int opt, const StageArgs& a, cudaStream_t st) {
  return launch_stage_order<4>(prec, opt, a, st);
}
}  // namespace sdg
