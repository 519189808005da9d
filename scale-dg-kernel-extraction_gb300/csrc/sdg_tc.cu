// Tensor-core form of the three directional contractions of
// tensorprod_divlike_dirXYZ (mod_dg_optr_kernel.f90:62-136; the per-order
// kernels of opt1 erb:228-344) in FP32 arithmetic, at p = 15 (Nq = 16).
//
// Batched over elements, each direction is a dense product: the lines of a
// direction are the rows of A (M = Nq^2 rows an element), the line's Nq
// values its K = Nq columns, and B(n, l) = D1D(n, l) gives the Nq outputs of
// a line as the N = Nq columns of D = A B^T.  One CTA of 128 threads runs
// tiles of 128 rows (half an element at Nq = 16):
//
//   * every thread loads its row's 16 values, splits each into a TF32 pair
//     hi = rna_tf32(x), lo = rna_tf32(x - hi), and stores both into shared
//     memory in the canonical K-major layout without swizzle (core matrices
//     of 8 rows x 16 bytes; K-adjacent core matrices 128 B apart, 8-row groups
//     512 B apart);
//   * one thread issues tcgen05.mma.cta_group::1.kind::tf32 (M = 128, N = 16,
//     K = 8) for A_hi B_hi + A_hi B_lo + A_lo B_hi over the two K halves --
//     six MMAs, FP32 accumulation in tensor memory (3xTF32, about FP32
//     accuracy) -- and commits them to an mbarrier;
//   * the CTA waits on the mbarrier (bounded: on a time-out it records an
//     error, waits once more, frees its tensor memory and stops), then each
//     warp reads its 32 rows of the accumulator with tcgen05.ld.32x32b.x16
//     and stores them.
//
// D1D's pair (hi, lo) is built once per CTA.  The CUDA-core form of the same
// FP32 contraction (divlike_f32_kernel) runs beside it for comparison.
#include <cuda_runtime.h>

#include <cstdint>

#include "sdg_internal.h"

using namespace sdg;

namespace {

constexpr int kTcRows = 128;      // M of one MMA tile
constexpr int kTcN = 16;          // N = K = Nq at p = 15
constexpr int kTcCols = 32;       // tensor-memory columns allocated (>= 32)
constexpr int kCoreK = 128;       // bytes between K-adjacent core matrices
constexpr int kCoreMN = 512;      // bytes between 8-row groups (16 K values a row)
constexpr long long kWaitLimit = 1LL << 24;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint32_t to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// Byte offset of (row, k) in the K-major no-swizzle layout.
__device__ __forceinline__ int kmajor_offset(int row, int k) {
  return (row >> 3) * kCoreMN + (k >> 2) * kCoreK + (row & 7) * 16 + (k & 3) * 4;
}

// Shared-memory matrix descriptor: start address, leading (K) and stride
// (M/N) byte offsets, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)((kCoreK >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((kCoreMN >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of kind::tf32: FP32 accumulator, TF32 A and B,
// both K-major, N = 16, M = 128.
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kTcN >> 3) << 17) |
                            ((uint32_t)(kTcRows >> 4) << 24);

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
      :
      : "r"(dtmem), "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(phase)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t phase) {
  for (long long it = 0; it < kWaitLimit; it++)
    if (mbar_try_wait(bar, phase)) return true;
  return false;
}

struct TcArgs {
  float* out[3];
  const float* in[3];
  const float* D;   // D1D(Nq, Nq), column-major
  long long nelem;
  int* err;
};

// A row R of direction d at element e: its 16 values are
// in[e*4096 + base(R) + l*strideK], its 16 results go to the same places.
__device__ __forceinline__ void row_geometry(int d, int R, int& base, int& stride) {
  if (d == 0) {
    base = 16 * R;
    stride = 1;
  } else if (d == 1) {
    base = (R & 15) + 256 * (R >> 4);
    stride = 16;
  } else {
    base = R;
    stride = 256;
  }
}

__global__ void __launch_bounds__(128) divlike_tc_kernel(const TcArgs a) {
  __shared__ __align__(1024) unsigned char sA[2][kTcRows * kTcN * 4];  // hi, lo
  __shared__ __align__(1024) unsigned char sB[2][kTcN * kTcN * 4];
  __shared__ __align__(8) unsigned long long mbar;
  __shared__ uint32_t tmem_base;
  const int tid = threadIdx.x, warp = tid >> 5;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :
                 : "r"(smem_addr(&tmem_base)), "r"(kTcCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&mbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // B = D1D as (n, l) rows, K-major: B(n, l) = D(n + 16 l)
  for (int t = tid; t < kTcN * kTcN; t += blockDim.x) {
    const int n = t & 15, l = t >> 4;
    const float x = a.D[n + 16 * l];
    const uint32_t hi = to_tf32(x);
    const uint32_t lo = to_tf32(x - __uint_as_float(hi));
    *reinterpret_cast<uint32_t*>(sB[0] + kmajor_offset(n, l)) = hi;
    *reinterpret_cast<uint32_t*>(sB[1] + kmajor_offset(n, l)) = lo;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;
  const uint32_t bar = smem_addr(&mbar);
  const uint32_t aHi = smem_addr(sA[0]), aLo = smem_addr(sA[1]);
  const uint32_t bHi = smem_addr(sB[0]), bLo = smem_addr(sB[1]);
  uint32_t phase = 0;
  const long long ntiles = a.nelem * 2 * 3;  // two 128-row halves a direction
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int d = (int)(tile % 3);
    const long long et = tile / 3;
    const long long e = et >> 1;
    const int R = (int)(et & 1) * kTcRows + tid;
    int base, stride;
    row_geometry(d, R, base, stride);
    const float* src = a.in[d] + e * 4096 + base;
#pragma unroll
    for (int l = 0; l < kTcN; l++) {
      const float x = src[l * stride];
      const uint32_t hi = to_tf32(x);
      const uint32_t lo = to_tf32(x - __uint_as_float(hi));
      *reinterpret_cast<uint32_t*>(sA[0] + kmajor_offset(tid, l)) = hi;
      *reinterpret_cast<uint32_t*>(sA[1] + kmajor_offset(tid, l)) = lo;
    }
    // the tensor cores read shared memory through the async proxy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (tid == 0) {
      // K halves: columns 0-7 and 8-15 are two core matrices apart
      uint32_t acc = 0;
      const uint32_t as[3] = {aHi, aHi, aLo}, bs[3] = {bHi, bLo, bHi};
#pragma unroll
      for (int term = 0; term < 3; term++)
#pragma unroll
        for (int kh = 0; kh < 2; kh++) {
          mma_tf32(tmem, smem_desc(as[term] + kh * 2 * kCoreK),
                   smem_desc(bs[term] + kh * 2 * kCoreK), acc);
          acc = 1;
        }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
          : "memory");
    }
    const bool done = mbar_wait_bounded(bar, phase);
    if (__syncthreads_or(!done)) {
      // the MMAs did not complete in time: record it, wait once more for
      // them before the tensor memory is released, and stop
      if (tid == 0) atomicExch(a.err, 1);
      mbar_wait_bounded(bar, phase);
      break;
    }
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // each warp reads its 32 lanes (rows) of the 128 x 16 accumulator
    uint32_t v[16];
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
        "%14,%15}, [%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
          "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
          "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    float* dst = a.out[d] + e * 4096 + base;
#pragma unroll
    for (int n = 0; n < kTcN; n++) dst[n * stride] = __uint_as_float(v[n]);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  }
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTcCols)
                 : "memory");
}

// The CUDA-core FP32 form: one thread per node and direction, D1D and the
// element's three inputs in shared memory, a running FP32 sum over l.
template <int NQ>
__global__ void __launch_bounds__(256) divlike_f32_kernel(const TcArgs a) {
  constexpr int NQ2 = NQ * NQ, NP = NQ2 * NQ;
  __shared__ float sD[NQ2];
  extern __shared__ float sF[];  // [3][NP]
  for (int t = threadIdx.x; t < NQ2; t += blockDim.x) sD[t] = a.D[t];
  for (long long e = blockIdx.x; e < a.nelem; e += gridDim.x) {
    __syncthreads();
    for (int t = threadIdx.x; t < 3 * NP; t += blockDim.x) {
      const int d = t / NP, n = t - d * NP;
      sF[t] = a.in[d][e * NP + n];
    }
    __syncthreads();
    for (int t = threadIdx.x; t < NP; t += blockDim.x) {
      const int i = t % NQ, j = (t / NQ) % NQ, k = t / NQ2;
      float sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
      for (int l = 0; l < NQ; l++) {
        sx = fmaf(sD[i + NQ * l], sF[l + NQ * j + NQ2 * k], sx);
        sy = fmaf(sD[j + NQ * l], sF[NP + i + NQ * l + NQ2 * k], sy);
        sz = fmaf(sD[k + NQ * l], sF[2 * NP + i + NQ * j + NQ2 * l], sz);
      }
      a.out[0][e * NP + t] = sx;
      a.out[1][e * NP + t] = sy;
      a.out[2][e * NP + t] = sz;
    }
  }
}

}  // namespace

extern "C" int sdg_tensorprod_divlike_dirXYZ_f32_dev(float* out_x, float* out_y, float* out_z,
                                                     const float* D1D, const float* in_x,
                                                     const float* in_y, const float* in_z,
                                                     int Nq, int nelem, int use_tensor_cores,
                                                     int* err_flag, void* stream) {
  if (Nq - 1 < 1 || Nq - 1 > kMaxOrder)
    return fail(SDG_ERR_UNSUPPORTED_ORDER, "PolyOrder %d outside 1..15", Nq - 1);
  if (use_tensor_cores && Nq != 16)
    return fail(SDG_ERR_UNSUPPORTED_ORDER,
                "the tensor-core contraction is built for Nq = 16 (p = 15), not Nq = %d", Nq);
  if (nelem < 0) return fail(SDG_ERR_INVALID_ARG, "nelem < 0");
  if (nelem == 0) return SDG_OK;
  if (!out_x || !out_y || !out_z || !D1D || !in_x || !in_y || !in_z || !err_flag)
    return fail(SDG_ERR_INVALID_ARG, "NULL device pointer");
  cudaStream_t st = as_stream(stream);
  TcArgs a{{out_x, out_y, out_z}, {in_x, in_y, in_z}, D1D, nelem, err_flag};
  if (use_tensor_cores) {
    const long long tiles = 6LL * nelem;
    const unsigned grid = (unsigned)(tiles < 152LL * 8 ? tiles : 152LL * 8);
    divlike_tc_kernel<<<grid, 128, 0, st>>>(a);
    SDG_CUDA_TRY(cudaGetLastError());
    return SDG_OK;
  }
  const unsigned grid = (unsigned)(nelem < 152LL * 16 ? nelem : 152LL * 16);
  const size_t smem = 3 * (size_t)Nq * Nq * Nq * sizeof(float);
  switch (Nq) {
#define SDG_F32_CASE(n)                                                                  \
  case n:                                                                                \
    SDG_TRY(set_kernel_smem((const void*)divlike_f32_kernel<n>, (int)smem, false));      \
    divlike_f32_kernel<n><<<grid, 256, smem, st>>>(a);                                   \
    break;
    SDG_F32_CASE(2) SDG_F32_CASE(3) SDG_F32_CASE(4) SDG_F32_CASE(5) SDG_F32_CASE(6)
    SDG_F32_CASE(7) SDG_F32_CASE(8) SDG_F32_CASE(9) SDG_F32_CASE(10) SDG_F32_CASE(11)
    SDG_F32_CASE(12) SDG_F32_CASE(13) SDG_F32_CASE(14) SDG_F32_CASE(15) SDG_F32_CASE(16)
#undef SDG_F32_CASE
    default:
      return fail(SDG_ERR_UNSUPPORTED_ORDER, "Nq %d", Nq);
  }
  SDG_CUDA_TRY(cudaGetLastError());
  return SDG_OK;
}
