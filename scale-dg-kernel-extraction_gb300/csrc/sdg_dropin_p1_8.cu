// Instantiations of the reference-shaped drop-in kernels for orders
// 1 2 3 4 5 6 7 8.
#include "sdg_dropin.cuh"

namespace sdg {
int dropin_p1(int what, int opt, const void* args, cudaStream_t st) {
  return dropin_order<1>(what, opt, args, st);
}
int dropin_p2(int what, int opt, const void* args, cudaStream_t st) {
  return dropin_order<2>(what, opt, args, st);
}
int dropin_p3(int what, int opt, const void* args, cudaStream_t st) {
  return dropin_order<3>(what, opt, args, st);
}
int dropin_p4(int what, int opt, const void* args, cudaStream_t st) {
  return dropin_order<4>(what, opt, args, st);
}
int dropin_p5(int what, int opt, const void* args, cudaStream_t st) {
  return dropin_order<5>(what, opt, args, st);
}
int dropin_p6(int what, int opt, const void* args, cudaStream_t st) {
  return dropin_order<6>(what, opt, args, st);
}
int dropin_p7(int what, int opt, const void* args, cudaStream_t st) {
  return dropin_order<7>(what, opt, args, st);
}
int dropin_p8(int what, int opt, const void* args, cudaStream_t st) {
  return dropin_order<8>(what, opt, args, st);
}
}  // namespace sdg
