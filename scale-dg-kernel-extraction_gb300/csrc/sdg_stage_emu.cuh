// Fused RK-stage kernel with emulated FP64 arithmetic (SDG_PREC_FP64_EMU).
//
// Same phases and data flow as stage_kernel (sdg_stage.cuh), but the flux,
// divergence and lift arithmetic runs in double-float (sdg_df.cuh) on the
// FP32 pipes.  The state stays FP64 in HBM, the RK combine runs in FP64, and
// the result matches the FP64 oracle to <= 1e-12 relative L2 per tendency
// (tested for p = 1..15).
//
// Algebraic folds (exact in real arithmetic, so only rounding changes):
//   - Escale_d is folded into the differentiation tables: Dd = Es_d * D1D;
//   - 0.5*Fscale of each face is folded into the lift table:
//     L'(n,f) = Lift_mat(n,f) * 0.5 * Fscale(f);
//   - the whole tendency of a node is one compensated dot product
//       dqdt = -( sum_l Dx(i,l) Fx(l,j,k) + sum_l Dy(j,l) Fy(i,l,k)
//               + sum_l Dz(k,l) Fz(i,j,l) + sum_f L'(n,f) g_f )
//     where g_f = qP velP - qM velM - alpha (qP - qM) is the unscaled upwind
//     flux (mod_advect3d_eq.f90:134-139) and F_d = q u_d (:181-183);
//   - the RK combine a*q0 + b*(q + dt*dqdt) (main.f90:70-71) is evaluated as
//     a*q0 + b*q + (b*dt)*dqdt with the last product in double-float.
// FP64 values enter through df_split and leave through f32_to_f64_bits, both
// integer/FP32 code, so the FP64 pipe (1/64 of the FP32 rate on GB300) only
// runs the two or three additions of the RK combine per node.
// The GENERAL / OPT1 summation orders have no meaning here: the compensated
// sum is more accurate than either.
#pragma once

#include "sdg_df.cuh"
#include "sdg_stage.cuh"

namespace sdg {

template <int P>
struct EmuCfg {
  static constexpr int EPB = StageCfg<P, float>::EPB;
  static constexpr int THREADS = StageCfg<P, float>::THREADS;
};

// floats of shared memory: D tables (3 axes x hi/lo), then per element
// q (2 NP), u, v, w (6 NP), face fluxes g (2 NFT)
template <int P>
constexpr size_t emu_smem_bytes() {
  using O = Ord<P>;
  return sizeof(float) * (size_t)(6 * O::NQ2 + EmuCfg<P>::EPB * (8 * O::NP + 2 * O::NFT));
}

template <int P>
__global__ void __launch_bounds__(EmuCfg<P>::THREADS) stage_emu_kernel(const StageArgs a) {
  using O = Ord<P>;
  constexpr int NQ = O::NQ, NQ2 = O::NQ2, NP = O::NP, NFP = O::NFP, NFT = O::NFT,
                EPB = EmuCfg<P>::EPB, T = EmuCfg<P>::THREADS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* sD = reinterpret_cast<float*>(smem_raw);  // [6][NQ2]: Dx hi, lo, Dy hi, lo, Dz hi, lo
  float* sqh = sD + 6 * NQ2;
  float* sql = sqh + EPB * NP;
  float* svh = sql + EPB * NP;  // [3][EPB*NP] hi planes of u, v, w
  float* svl = svh + 3 * EPB * NP;
  float* sgh = svl + 3 * EPB * NP;
  float* sgl = sgh + EPB * NFT;

  const long long eb = a.elem_begin + (long long)blockIdx.x * EPB;
  const long long eend = a.elem_begin + a.elem_count;
  const int nloc = (int)((eend - eb) < EPB ? (eend - eb) : EPB);
  if (nloc <= 0) return;
  const double* __restrict__ qin = a.q_in;
  const float2* __restrict__ gu = static_cast<const float2*>(a.u);
  const float2* __restrict__ gv = static_cast<const float2*>(a.v);
  const float2* __restrict__ gw = static_cast<const float2*>(a.w);
  const long long g0 = eb * NP;
  constexpr int SV = EPB * NP;  // stride between the u, v, w planes

  // phase 0: stage state (split to double-float) and velocity
  for (int t = threadIdx.x; t < 6 * NQ2; t += T) sD[t] = static_cast<const float*>(a.D)[t];
  for (int t = threadIdx.x; t < nloc * NP; t += T) {
    const dfl q = df_split(qin[g0 + t]);
    sqh[t] = q.hi;
    sql[t] = q.lo;
    const float2 uu = gu[g0 + t], vv = gv[g0 + t], ww = gw[g0 + t];
    svh[t] = uu.x;
    svl[t] = uu.y;
    svh[SV + t] = vv.x;
    svl[SV + t] = vv.y;
    svh[2 * SV + t] = ww.x;
    svl[2 * SV + t] = ww.y;
  }
  __syncthreads();

  // phase 1: unscaled upwind flux g on every face node
  for (int t = threadIdx.x; t < nloc * NFT; t += T) {
    const int le = t / NFT;
    const int r = t - le * NFT;
    const int f = r / NFP;
    const int fp = r - f * NFP;
    int nM, nP, axis, sg;
    face_nodes<NQ>(f, fp % NQ, fp / NQ, nM, nP, axis, sg);
    const long long eP = neighbor(a.box, eb + le, f);
    const long long gP = eP * NP + nP;
    const int iM = le * NP + nM;
    const float sgn = (float)sg;
    const dfl qM = df_make(sqh[iM], sql[iM]);
    const dfl velM = df_make(sgn * svh[axis * SV + iM], sgn * svl[axis * SV + iM]);
    const dfl qP = df_split(qin[gP]);
    const float2 vp = ((axis == 0) ? gu : (axis == 1) ? gv : gw)[gP];
    const dfl velP = df_make(sgn * vp.x, sgn * vp.y);
    const dfl alpha = df_scale2(df_abs(df_add(velP, velM)), 0.5f);
    const dfl jump = df_sub(qP, qM);
    dacc A = dacc_zero();
    dacc_fma(A, qP, velP);
    dacc_fma(A, df_neg(qM), velM);
    dacc_fma(A, df_neg(alpha), jump);
    const dfl gflux = dacc_result(A);
    sgh[le * NFT + r] = gflux.hi;
    sgl[le * NFT + r] = gflux.lo;
  }
  __syncthreads();

  // phase 2: F_d = q * u_d in place
  for (int t = threadIdx.x; t < nloc * NP; t += T) {
    const dfl q = df_make(sqh[t], sql[t]);
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const dfl F = df_mul(q, df_make(svh[d * SV + t], svl[d * SV + t]));
      svh[d * SV + t] = F.hi;
      svl[d * SV + t] = F.lo;
    }
  }
  __syncthreads();

  // phase 3: one compensated dot product per node, then the RK combine
  const float* __restrict__ Lh = static_cast<const float*>(a.Lift);
  const float* __restrict__ Ll = Lh + 6 * NP;
  const dfl c_dt = df_make(a.cdt_hi, a.cdt_lo);  // b*dt split on the host
  for (int t = threadIdx.x; t < nloc * NP; t += T) {
    const int le = t / NP;
    const int n = t - le * NP;
    const int i = n % NQ;
    const int j = (n / NQ) % NQ;
    const int k = n / NQ2;
    const int base = le * NP;
    dacc A = dacc_zero();
#pragma unroll
    for (int l = 0; l < NQ; l++) {
      const int fi = base + l + j * NQ + k * NQ2;
      dacc_fma(A, df_make(sD[0 * NQ2 + l * NQ + i], sD[1 * NQ2 + l * NQ + i]),
               df_make(svh[fi], svl[fi]));
    }
#pragma unroll
    for (int l = 0; l < NQ; l++) {
      const int fi = SV + base + i + l * NQ + k * NQ2;
      dacc_fma(A, df_make(sD[2 * NQ2 + l * NQ + j], sD[3 * NQ2 + l * NQ + j]),
               df_make(svh[fi], svl[fi]));
    }
#pragma unroll
    for (int l = 0; l < NQ; l++) {
      const int fi = 2 * SV + base + i + j * NQ + l * NQ2;
      dacc_fma(A, df_make(sD[4 * NQ2 + l * NQ + k], sD[5 * NQ2 + l * NQ + k]),
               df_make(svh[fi], svl[fi]));
    }
    const int gb = le * NFT;
    const int fidx[6] = {i + k * NQ, NFP + j + k * NQ, 2 * NFP + i + k * NQ,
                         3 * NFP + j + k * NQ, 4 * NFP + i + j * NQ, 5 * NFP + i + j * NQ};
#pragma unroll
    for (int f = 0; f < 6; f++)
      dacc_fma(A, df_make(__ldg(Lh + n + f * NP), __ldg(Ll + n + f * NP)),
               df_make(sgh[gb + fidx[f]], sgl[gb + fidx[f]]));
    const dfl dq = df_neg(dacc_result(A));
    const long long g = g0 + t;
    // FP32 -> FP64 widening by bit manipulation keeps the FP64 pipe for the
    // additions of the RK combine only
    if (a.tend_only) {
      a.q_out[g] = f32_to_f64_bits(dq.hi) + f32_to_f64_bits(dq.lo);
    } else {
      const dfl inc = df_mul(c_dt, dq);  // (b*dt)*dqdt
      const double ih = f32_to_f64_bits(inc.hi), il = f32_to_f64_bits(inc.lo);
      const double qv = qin[g];
      double r = ((a.b == 1.0) ? qv + ih : fma(a.b, qv, ih)) + il;
      if (a.a != 0.0) r = fma(a.a, a.q0[g], r);
      a.q_out[g] = r;
    }
  }
}

template <int P>
int launch_stage_emu_impl(const StageArgs& a, cudaStream_t st) {
  using C = EmuCfg<P>;
  constexpr size_t smem = emu_smem_bytes<P>();
  SDG_CUDA_TRY(cudaFuncSetAttribute(stage_emu_kernel<P>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const long long nblk = (a.elem_count + C::EPB - 1) / C::EPB;
  if (nblk <= 0) return SDG_OK;
  if (nblk > 0x7fffffffLL) return fail(SDG_ERR_INVALID_ARG, "too many elements");
  stage_emu_kernel<P><<<(unsigned)nblk, C::THREADS, smem, st>>>(a);
  SDG_CUDA_TRY(cudaGetLastError());
  return SDG_OK;
}

}  // namespace sdg
