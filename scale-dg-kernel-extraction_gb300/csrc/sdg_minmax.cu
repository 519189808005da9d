// Device min/max of an FP64 field: the diagnostic the reference's time loop
// prints every output_interval steps (main.f90:76-79, minval/maxval of
// q(:,1:Ne)).
//
// Each double is mapped to an unsigned 64-bit key whose integer order is the
// IEEE total order (negative values: all bits flipped; others: sign bit set).
// Comparisons then run on the integer ALUs instead of the 1/64-rate FP64 pipe,
// the result is exact and independent of the reduction order, and one 64-bit
// atomicMin / atomicMax per block combines the blocks.  A record's keys are
// reset by two memsets (0xFF.. for min, 0 for max) before its reduction.
#include <cuda_runtime.h>

#include <cstring>

#include "sdg_internal.h"

namespace sdg {

namespace {

__device__ __forceinline__ unsigned long long order_key(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

__device__ __forceinline__ unsigned long long umin64(unsigned long long a, unsigned long long b) {
  return a < b ? a : b;
}
__device__ __forceinline__ unsigned long long umax64(unsigned long long a, unsigned long long b) {
  return a > b ? a : b;
}

constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads)
    minmax_kernel(const double* __restrict__ q, long long n, unsigned long long* kmin,
                  unsigned long long* kmax) {
  unsigned long long lo = ~0ull, hi = 0ull;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  // pairs of doubles with 16-byte loads when q is 16-byte aligned
  if ((reinterpret_cast<uintptr_t>(q) & 15) == 0) {
    const double2* q2 = reinterpret_cast<const double2*>(q);
    const long long n2 = n >> 1;
    for (long long i = t0; i < n2; i += stride) {
      const double2 v = __ldg(q2 + i);
      const unsigned long long a = order_key(v.x), b = order_key(v.y);
      lo = umin64(lo, umin64(a, b));
      hi = umax64(hi, umax64(a, b));
    }
    if (t0 == 0 && (n & 1)) {
      const unsigned long long a = order_key(q[n - 1]);
      lo = umin64(lo, a);
      hi = umax64(hi, a);
    }
  } else {
    for (long long i = t0; i < n; i += stride) {
      const unsigned long long a = order_key(q[i]);
      lo = umin64(lo, a);
      hi = umax64(hi, a);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = umin64(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = umax64(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  __shared__ unsigned long long s_lo[kThreads / 32], s_hi[kThreads / 32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    s_lo[warp] = lo;
    s_hi[warp] = hi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < kThreads / 32; k++) {
      lo = umin64(lo, s_lo[k]);
      hi = umax64(hi, s_hi[k]);
    }
    atomicMin(kmin, lo);
    atomicMax(kmax, hi);
  }
}

}  // namespace

double minmax_key_to_double(unsigned long long k) {
  const unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  double x;
  std::memcpy(&x, &b, 8);
  return x;
}

int minmax_launch(const double* q, long long n, unsigned long long* kmin, unsigned long long* kmax,
                  cudaStream_t st) {
  SDG_CUDA_TRY(cudaMemsetAsync(kmin, 0xff, sizeof(unsigned long long), st));
  SDG_CUDA_TRY(cudaMemsetAsync(kmax, 0x00, sizeof(unsigned long long), st));
  if (n <= 0) return SDG_OK;
  long long nb = ((n + 1) / 2 + kThreads - 1) / kThreads;
  if (nb > 152LL * 8) nb = 152LL * 8;
  minmax_kernel<<<(unsigned)(nb > 0 ? nb : 1), kThreads, 0, st>>>(q, n, kmin, kmax);
  SDG_CUDA_TRY(cudaGetLastError());
  return SDG_OK;
}

}  // namespace sdg

using namespace sdg;

extern "C" int sdg_minmax_dev(const double* q, long long n, double* qmin, double* qmax,
                              void* stream) {
  if (!q || !qmin || !qmax) return fail(SDG_ERR_INVALID_ARG, "NULL argument");
  if (n < 1) return fail(SDG_ERR_INVALID_ARG, "n < 1");
  SDG_TRY(require_device());
  cudaStream_t st = as_stream(stream);
  unsigned long long* keys = nullptr;
  SDG_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&keys), 2 * sizeof(unsigned long long), st));
  unsigned long long hk[2] = {0, 0};
  int rc = minmax_launch(q, n, keys, keys + 1, st);
  cudaError_t e = cudaSuccess;
  if (rc == SDG_OK) e = cudaMemcpyAsync(hk, keys, sizeof(hk), cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(keys, st);
  if (rc != SDG_OK) return rc;
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "sdg_minmax_dev", __FILE__, __LINE__);
  *qmin = minmax_key_to_double(hk[0]);
  *qmax = minmax_key_to_double(hk[1]);
  return SDG_OK;
}
