// Instantiations of the reference-shaped drop-in kernels for orders
// 9 10 11 12 13 14 15.
#include "sdg_dropin.cuh"

namespace sdg {
int dropin_p9(int what, int opt, const void* args, cudaStream_t st) {
  return dropin_order<9>(what, opt, args, st);
}
int dropin_p10(int what, int opt, const void* args, cudaStream_t st) {
  return dropin_order<10>(what, opt, args, st);
}
int dropin_p11(int what, int opt, const void* args, cudaStream_t st) {
  return dropin_order<11>(what, opt, args, st);
}
int dropin_p12(int what, int opt, const void* args, cudaStream_t st) {
  return dropin_order<12>(what, opt, args, st);
}
int dropin_p13(int what, int opt, const void* args, cudaStream_t st) {
  return dropin_order<13>(what, opt, args, st);
}
int dropin_p14(int what, int opt, const void* args, cudaStream_t st) {
  return dropin_order<14>(what, opt, args, st);
}
int dropin_p15(int what, int opt, const void* args, cudaStream_t st) {
  return dropin_order<15>(what, opt, args, st);
}
}  // namespace sdg
