// Line-blocked fused stage body for the FP32-compute / FP64-state form.
//
// Same numerics as stage_block<P, float, float, SPLIT3> (sdg_stage.cuh): FP32
// flux, divergence and lift, FP64 RK state; the per-node combine keeps the
// reference's order ((Ex dx + Ey dy) + Ez dz) + lift (mod_advect3d_eq.f90:
// 194-198).  The work is arranged for GB300's shared-memory bandwidth: one
// thread owns a line of Nq nodes along an axis and keeps its Nq volume fluxes
// in registers, so each shared-memory load feeds Nq FMAs (the node-per-thread
// form needs two loads per FMA).  Per element, three planes hold F_x, F_y,
// F_z, each laid out line-major for its own axis with one pad slot per line
// against bank conflicts; the x plane then holds the running combine.
//   0  F_d = q u_d into the planes; 1 upwind face fluxes (own and neighbour
//   values read from global memory, where the staging loads left them in
//   L1/L2); 3x, 3y, 3z contractions per line; 3z adds the lift, finishes
//   the combine and writes the RK update.
// nloc and the block size are runtime values, so the batched persistent
// kernel runs the same body with any elements-per-block choice.
#pragma once

#include "sdg_stage.cuh"

namespace sdg {

template <int P>
struct F32Cfg {
  static constexpr int NQ2 = (P + 1) * (P + 1);
  static constexpr int EPB = (256 / NQ2) > 0 ? (256 / NQ2) : 1;
  static constexpr int THREADS = ((EPB * NQ2 + 31) / 32) * 32;
  static constexpr int PADL = P + 2;
  static constexpr int PLANE = PADL * NQ2;
};

template <int P>
__host__ __device__ constexpr size_t f32_block_smem(int nloc) {
  using C = F32Cfg<P>;
  return sizeof(float) * (size_t)(C::NQ2 + nloc * (3 * C::PLANE + 6 * C::NQ2));
}

// sum_l d[l*NQ] * f[l], GENERAL running order or the OPT1 three-way split.
template <int NQ, bool SPLIT3>
__device__ __forceinline__ float line_reg_sum(const float* __restrict__ d, const float (&f)[NQ]) {
  if constexpr (!SPLIT3) {
    float s = d[0] * f[0];
#pragma unroll
    for (int l = 1; l < NQ; l++) s = fmaf(d[l * NQ], f[l], s);
    return s;
  } else {
    constexpr int D3 = (2 * NQ + 3) / 6;  // round(NQ/3.0) for NQ in 9..16
    float t1 = d[0] * f[0];
#pragma unroll
    for (int l = 1; l < D3; l++) t1 = fmaf(d[l * NQ], f[l], t1);
    float t2 = d[D3 * NQ] * f[D3];
#pragma unroll
    for (int l = D3 + 1; l < 2 * D3; l++) t2 = fmaf(d[l * NQ], f[l], t2);
    float t3 = d[2 * D3 * NQ] * f[2 * D3];
#pragma unroll
    for (int l = 2 * D3 + 1; l < NQ; l++) t3 = fmaf(d[l * NQ], f[l], t3);
    return (t1 + t2) + t3;
  }
}

template <int P, bool SPLIT3>
__device__ __forceinline__ void stage_block_f32(const StageArgs& a, long long eb, int nloc,
                                                unsigned char* smem) {
  using O = Ord<P>;
  using C = F32Cfg<P>;
  constexpr int NQ = O::NQ, NQ2 = O::NQ2, NP = O::NP, NFP = O::NFP, NFT = O::NFT,
                PADL = C::PADL, PLANE = C::PLANE;
  const int T = blockDim.x;
  float* sD = reinterpret_cast<float*>(smem);  // D(i,l) at l*NQ + i
  float* sPl = sD + NQ2;                       // [nloc][3][PLANE]
  float* sg = sPl + nloc * 3 * PLANE;          // [nloc][NFT]
  const double* __restrict__ qin = a.q_in;
  const float* __restrict__ gu = static_cast<const float*>(a.u);
  const float* __restrict__ gv = static_cast<const float*>(a.v);
  const float* __restrict__ gw = static_cast<const float*>(a.w);
  const long long g0 = eb * NP;

  // phase 0
  for (int t = threadIdx.x; t < NQ2; t += T) sD[t] = static_cast<const float*>(a.D)[t];
  for (int t = threadIdx.x; t < nloc * NP; t += T) {
    const int le = t / NP;
    const int n = t - le * NP;
    const int i = n % NQ, j = (n / NQ) % NQ, k = n / NQ2;
    const float qq = to_ct<float>(qin[g0 + t]);
    float* pl = sPl + le * 3 * PLANE;
    pl[i + PADL * (j + NQ * k)] = qq * gu[g0 + t];
    pl[PLANE + j + PADL * (i + NQ * k)] = qq * gv[g0 + t];
    pl[2 * PLANE + k + PADL * (i + NQ * j)] = qq * gw[g0 + t];
  }
  // phase 1: element-boundary flux (mod_advect3d_eq.f90:116-140)
  for (int t = threadIdx.x; t < nloc * NFT; t += T) {
    const int le = t / NFT;
    const int r = t - le * NFT;
    const int f = r / NFP;
    const int fp = r - f * NFP;
    int nM, nP, axis, sgi;
    face_nodes<NQ>(f, fp % NQ, fp / NQ, nM, nP, axis, sgi);
    const long long eP = neighbor(a.box, eb + le, f);
    const long long gM = (eb + le) * NP + nM, gP = eP * NP + nP;
    const float* gvel = (axis == 0) ? gu : (axis == 1) ? gv : gw;
    const float sgn = (float)sgi;
    const float qM = to_ct<float>(qin[gM]), qP = to_ct<float>(qin[gP]);
    const float velM = sgn * gvel[gM], velP = sgn * gvel[gP];
    const float alpha = 0.5f * fabsf(velP + velM);
    const float fs = (float)a.box.Fs[axis];
    sg[le * NFT + r] = (0.5f * fs) * ((qP * velP - qM * velM) - alpha * (qP - qM));
  }
  __syncthreads();

  const float Ex = (float)a.box.Es[0], Ey = (float)a.box.Es[1], Ez = (float)a.box.Es[2];
  // 3x: line (j, k); Ex * dx goes to the x plane in place
  for (int r = threadIdx.x; r < nloc * NQ2; r += T) {
    const int le = r / NQ2, line = r - le * NQ2;
    float* pl = sPl + le * 3 * PLANE + PADL * line;
    float F[NQ];
#pragma unroll
    for (int l = 0; l < NQ; l++) F[l] = pl[l];
#pragma unroll
    for (int i = 0; i < NQ; i++) pl[i] = Ex * line_reg_sum<NQ, SPLIT3>(sD + i, F);
  }
  __syncthreads();
  // 3y: line (i, k); acc = Ex dx + Ey dy
  for (int r = threadIdx.x; r < nloc * NQ2; r += T) {
    const int le = r / NQ2, line = r - le * NQ2;
    const int i = line % NQ, k = line / NQ;
    float* pl = sPl + le * 3 * PLANE;
    float F[NQ];
#pragma unroll
    for (int l = 0; l < NQ; l++) F[l] = pl[PLANE + PADL * line + l];
#pragma unroll
    for (int j = 0; j < NQ; j++) {
      float& acc = pl[i + PADL * (j + NQ * k)];
      acc = acc + Ey * line_reg_sum<NQ, SPLIT3>(sD + j, F);
    }
  }
  __syncthreads();
  // 3z: line (i, j); + Ez dz, + lift, RK combine, store
  const float* __restrict__ L = static_cast<const float*>(a.Lift);
  for (int r = threadIdx.x; r < nloc * NQ2; r += T) {
    const int le = r / NQ2, line = r - le * NQ2;
    const int i = line % NQ, j = line / NQ;
    const float* pl = sPl + le * 3 * PLANE;
    const float* fl = sg + le * NFT;
    float F[NQ];
#pragma unroll
    for (int l = 0; l < NQ; l++) F[l] = pl[2 * PLANE + PADL * line + l];
#pragma unroll 2
    for (int k = 0; k < NQ; k++) {
      const float acc = pl[i + PADL * (j + NQ * k)] + Ez * line_reg_sum<NQ, SPLIT3>(sD + k, F);
      const int n = i + j * NQ + k * NQ2;
      const float lf = lift_node<P>(L + n, fl, i, j, k);
      const float dq = -(acc + lf);
      const long long g = (eb + le) * NP + n;
      if (a.tend_only) {
        a.q_out[g] = f32_to_f64_bits(dq);
      } else {
        // the increment (b*dt)*dqdt is an FP32 product widened by bits; the
        // state combination a*q0 + b*q + increment stays FP64
        const double inc = f32_to_f64_bits(a.cdt_hi * dq);
        const double qv = qin[g];
        double rq = (a.b == 1.0) ? qv + inc : fma(a.b, qv, inc);
        if (a.a != 0.0) rq = fma(a.a, a.q0[g], rq);
        a.q_out[g] = rq;
      }
    }
  }
}

template <int P, bool SPLIT3>
__global__ void __launch_bounds__(F32Cfg<P>::THREADS) stage_f32_kernel(const StageArgs a) {
  constexpr int EPB = F32Cfg<P>::EPB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const long long eb = a.elem_begin + (long long)blockIdx.x * EPB;
  const long long eend = a.elem_begin + a.elem_count;
  const int nloc = (int)((eend - eb) < EPB ? (eend - eb) : EPB);
  if (nloc <= 0) return;
  stage_block_f32<P, SPLIT3>(a, eb, nloc, smem_raw);
}

template <int P, bool SPLIT3>
int launch_stage_f32_impl(const StageArgs& a, cudaStream_t st) {
  using C = F32Cfg<P>;
  constexpr size_t smem = f32_block_smem<P>(C::EPB);
  SDG_CUDA_TRY(cudaFuncSetAttribute(stage_f32_kernel<P, SPLIT3>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const long long nblk = (a.elem_count + C::EPB - 1) / C::EPB;
  if (nblk <= 0) return SDG_OK;
  if (nblk > 0x7fffffffLL) return fail(SDG_ERR_INVALID_ARG, "too many elements");
  stage_f32_kernel<P, SPLIT3><<<(unsigned)nblk, C::THREADS, smem, st>>>(a);
  SDG_CUDA_TRY(cudaGetLastError());
  return SDG_OK;
}

}  // namespace sdg
