// Double-float arithmetic: an FP64 value carried as an unevaluated sum of two
// FP32 numbers hi + lo (|lo| <= ulp(hi)/2), computed on the FP32 pipes.
//
// GB300 executes FP64 arithmetic at 1/64 of the FP32 rate (measured: 1.2
// TFLOP/s DFMA against 75 TFLOP/s FFMA), so the emulated FP64 stage kernel does
// its flux, divergence and lift arithmetic with these error-free
// transformations and keeps FP64 only for the state and the RK combine.
// Published building blocks:
//   TwoSum (Knuth, TAOCP vol. 2; Moller 1965): s + e = a + b exactly, 6 ops;
//   Fast2Sum (Dekker 1971): same when |a| >= |b|, 3 ops;
//   TwoProd with FMA: p + e = a * b exactly, 2 ops;
//   compensated dot product Dot2 (Ogita, Rump, Oishi 2005), here with
//   double-float operands: the running high sum goes through TwoSum and all
//   error and cross terms collect in a second FP32 accumulator.
// Precision: about 48 significant bits (two 24-bit significands).
//
// Every FP32 operation uses a round-to-nearest intrinsic on the device (no
// contraction into FMA unless written as one) and plain operations compiled
// without contraction on the host, so a host build computes the same bits.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#if defined(__CUDA_ARCH__)
#define SDG_HD __host__ __device__ __forceinline__
#define DFM(a, b) __fmul_rn((a), (b))
#define DFA(a, b) __fadd_rn((a), (b))
#define DFS(a, b) __fsub_rn((a), (b))
#define DFF(a, b, c) __fmaf_rn((a), (b), (c))
#elif defined(__CUDACC__)
#define SDG_HD __host__ __device__ inline
#define DFM(a, b) ((a) * (b))
#define DFA(a, b) ((a) + (b))
#define DFS(a, b) ((a) - (b))
#define DFF(a, b, c) std::fmaf((a), (b), (c))
#else
#define SDG_HD inline
#define DFM(a, b) ((a) * (b))
#define DFA(a, b) ((a) + (b))
#define DFS(a, b) ((a) - (b))
#define DFF(a, b, c) std::fmaf((a), (b), (c))
#endif

namespace sdg {

struct dfl {
  float hi, lo;
};

SDG_HD dfl df_make(float hi, float lo) {
  dfl r;
  r.hi = hi;
  r.lo = lo;
  return r;
}

// ---- bit casts ---------------------------------------------------------------
SDG_HD uint32_t f2u(float f) {
#if defined(__CUDA_ARCH__)
  return (uint32_t)__float_as_uint(f);
#else
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
#endif
}
SDG_HD float u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f;
  std::memcpy(&f, &u, 4);
  return f;
#endif
}
SDG_HD void d2words(double x, uint32_t& hi, uint32_t& lo) {
#if defined(__CUDA_ARCH__)
  hi = (uint32_t)__double2hiint(x);
  lo = (uint32_t)__double2loint(x);
#else
  uint64_t b;
  std::memcpy(&b, &x, 8);
  hi = (uint32_t)(b >> 32);
  lo = (uint32_t)b;
#endif
}
SDG_HD double words2d(uint32_t hi, uint32_t lo) {
#if defined(__CUDA_ARCH__)
  return __hiloint2double((int)hi, (int)lo);
#else
  const uint64_t b = ((uint64_t)hi << 32) | lo;
  double x;
  std::memcpy(&x, &b, 8);
  return x;
#endif
}

// hi = RN32(x); lo = RN32(x - hi).  x - hi is exact in FP64 (Sterbenz), so the
// pair carries x to within 2^-48 |x|.  This form runs its conversions and the
// subtraction on the FP64 pipe; df_split below gives the same kind of pair with
// integer and FP32 operations only.
SDG_HD dfl df_from_double(double x) {
  const float hi = (float)x;
  const float lo = (float)(x - (double)hi);
  return df_make(hi, lo);
}

// hi + lo has at most 48 significant bits, so the FP64 sum is exact.
SDG_HD double df_to_double(dfl a) { return (double)a.hi + (double)a.lo; }

// Exact FP32 -> FP64 widening from the bit pattern (integer operations only).
// Zero and FP32 subnormals (which df_split never produces) map to zero.
SDG_HD double f32_to_f64_bits(float f) {
  const uint32_t u = f2u(f);
  const uint32_t mag = u & 0x7FFFFFFFu;
  // exponent rebias 127 -> 1023 is +896 in the exponent field: (896 << 20)
  const uint32_t hi = (mag < 0x00800000u) ? (u & 0x80000000u)
                                          : ((u & 0x80000000u) | ((mag >> 3) + 0x38000000u));
  const uint32_t lo = (mag < 0x00800000u) ? 0u : (u << 29);
  return words2d(hi, lo);
}

// Splits an FP64 value into hi + lo with integer and FP32 operations only (no
// FP64 instruction): hi is x rounded to 24 significant bits (round half up on
// the magnitude), the remainder x - hi is an exact signed 29-bit multiple of
// the double's last-place unit, and lo = RN32(x - hi).  |x - (hi + lo)| <=
// 2^-48 |x| for 2^-74 <= |x| < 2^128; below 2^-74 lo is dropped (hi keeps 24
// bits) and below 2^-126 the pair is zero.
SDG_HD dfl df_split(double x) {
  uint32_t xh, xl;
  d2words(x, xh, xl);
  const uint32_t sign = xh & 0x80000000u;
  const uint32_t mag_hi = xh & 0x7FFFFFFFu;
  const int E = (int)(mag_hi >> 20);  // biased FP64 exponent
  if (E < 897) return df_make(0.0f, 0.0f);
  // magnitude rounded to 24 bits: truncated FP32 pattern plus the first
  // dropped bit (a carry into the exponent field is the correct rounding)
  const uint32_t rb = (xl >> 28) & 1u;
  const uint32_t trunc = ((mag_hi - 0x38000000u) << 3) | (xl >> 29);
  const float hi = u2f(sign | (trunc + rb));
  if (E < 949) return df_make(hi, 0.0f);
  // remainder in units of 2^(E-1075): r - rb*2^29, in [-2^28, 2^28)
  const int32_t rr = (int32_t)(xl & 0x1FFFFFFFu) - (int32_t)(rb << 29);
  const int32_t nh = rr >> 6;  // floor division by 64, |nh| <= 2^22
  const int32_t nl = rr & 63;
  // exact small-integer to FP32 conversions with the 1.5*2^23 / 2^23 constants
  const float fnh = DFS(u2f((uint32_t)(0x4B400000 + nh)), 12582912.0f);
  const float fnl = DFS(u2f(0x4B000000u | (uint32_t)nl), 8388608.0f);
  const float m = DFF(fnh, 64.0f, fnl);  // RN32(rr)
  const float scale = u2f(((uint32_t)(E - 948) << 23) | sign);  // +-2^(E-1075)
  return df_make(hi, DFM(m, scale));
}

SDG_HD dfl two_sum(float a, float b) {
  const float s = DFA(a, b);
  const float bb = DFS(s, a);
  const float e = DFA(DFS(a, DFS(s, bb)), DFS(b, bb));
  return df_make(s, e);
}

SDG_HD dfl fast_two_sum(float a, float b) {
  const float s = DFA(a, b);
  return df_make(s, DFS(b, DFS(s, a)));
}

SDG_HD dfl df_neg(dfl a) { return df_make(-a.hi, -a.lo); }

SDG_HD dfl df_scale2(dfl a, float pow2) {  // exact for a power of two
  return df_make(DFM(a.hi, pow2), DFM(a.lo, pow2));
}

SDG_HD dfl df_abs(dfl a) { return (a.hi < 0.0f) ? df_neg(a) : a; }

SDG_HD dfl df_add(dfl a, dfl b) {
  dfl s = two_sum(a.hi, b.hi);
  const float e = DFA(s.lo, DFA(a.lo, b.lo));
  return fast_two_sum(s.hi, e);
}

SDG_HD dfl df_sub(dfl a, dfl b) { return df_add(a, df_neg(b)); }

// a*b to ~2^-48 relative (the lo*lo term, 2^-48 below, is dropped).
SDG_HD dfl df_mul(dfl a, dfl b) {
  const float p = DFM(a.hi, b.hi);
  float e = DFF(a.hi, b.hi, -p);
  e = DFF(a.hi, b.lo, e);
  e = DFF(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}

// Compensated accumulator of products: s is the running high sum, c collects
// the exact product errors, the exact addition errors and the cross terms.
struct dacc {
  float s, c;
};

SDG_HD dacc dacc_zero() {
  dacc r;
  r.s = 0.0f;
  r.c = 0.0f;
  return r;
}

SDG_HD void dacc_fma(dacc& A, dfl a, dfl b) {
  const float p = DFM(a.hi, b.hi);
  const float pe = DFF(a.hi, b.hi, -p);
  const dfl t = two_sum(A.s, p);
  A.s = t.hi;
  A.c = DFA(A.c, DFA(pe, t.lo));
  A.c = DFF(a.hi, b.lo, A.c);
  A.c = DFF(a.lo, b.hi, A.c);
}

SDG_HD void dacc_add(dacc& A, dfl a) {
  const dfl t = two_sum(A.s, a.hi);
  A.s = t.hi;
  A.c = DFA(A.c, DFA(t.lo, a.lo));
}

SDG_HD dfl dacc_result(dacc A) { return two_sum(A.s, A.c); }

}  // namespace sdg
