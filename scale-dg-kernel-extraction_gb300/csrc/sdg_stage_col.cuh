// Column-blocked fused stage body for the FP32-compute / FP64-state form.
//
// Same numerics as stage_block<P, float, float, SPLIT3> (sdg_stage.cuh): FP32
// flux, divergence and lift, FP64 RK state, and the reference's combine order
// ((Ex dx + Ey dy) + Ez dz) + lift (mod_advect3d_eq.f90:194-198).  The work is
// arranged for the shared-memory bandwidth: one thread owns an (i, j) column
// of Nq nodes along z and
//   - keeps the column's z-fluxes F_z(i,j,:) in registers, so the z
//     contraction reads only D(k,l) (one broadcast load per FMA);
//   - keeps the rows D(i,:) and D(j,:) in registers, so the x and y
//     contractions read only the fluxes F_x(:,j,k) and F_y(i,:,k) from shared
//     memory (one load per FMA instead of two);
//   - walks k, so the node index is a loop counter rather than a division.
// Shared memory per element: q, F_x, F_y (Np each) and the face fluxes.
#pragma once

#include "sdg_stage.cuh"

namespace sdg {

template <int P>
__host__ __device__ constexpr size_t col_block_smem(int nloc) {
  using O = Ord<P>;
  return sizeof(float) * (size_t)(O::NQ2 + nloc * (3 * O::NP + O::NFT)) + sizeof(int) * 6 * nloc;
}

template <int P, bool SPLIT3>
__device__ __forceinline__ float reg_line_sum(const float (&d)[P + 1], const float* __restrict__ f,
                                              int stride) {
  constexpr int NQ = P + 1;
  if constexpr (!SPLIT3) {
    float s = d[0] * f[0];
#pragma unroll
    for (int l = 1; l < NQ; l++) s = fmaf(d[l], f[l * stride], s);
    return s;
  } else {
    constexpr int D3 = (2 * NQ + 3) / 6;  // round(NQ/3.0) for NQ in 9..16
    float t1 = d[0] * f[0];
#pragma unroll
    for (int l = 1; l < D3; l++) t1 = fmaf(d[l], f[l * stride], t1);
    float t2 = d[D3] * f[D3 * stride];
#pragma unroll
    for (int l = D3 + 1; l < 2 * D3; l++) t2 = fmaf(d[l], f[l * stride], t2);
    float t3 = d[2 * D3] * f[2 * D3 * stride];
#pragma unroll
    for (int l = 2 * D3 + 1; l < NQ; l++) t3 = fmaf(d[l], f[l * stride], t3);
    return (t1 + t2) + t3;
  }
}

template <int P, bool SPLIT3>
__device__ __forceinline__ void stage_block_col(const StageArgs& a, long long eb, int nloc,
                                                unsigned char* smem) {
  using O = Ord<P>;
  constexpr int NQ = O::NQ, NQ2 = O::NQ2, NP = O::NP, NFP = O::NFP, NFT = O::NFT;
  const int T = blockDim.x;
  float* sD = reinterpret_cast<float*>(smem);  // D(i,l) at l*NQ + i
  float* sq = sD + NQ2;
  float* sfx = sq + nloc * NP;
  float* sfy = sfx + nloc * NP;
  float* sf = sfy + nloc * NP;
  int* snb = reinterpret_cast<int*>(sf + nloc * NFT);
  const double* __restrict__ qin = a.q_in;
  const float* __restrict__ gu = static_cast<const float*>(a.u);
  const float* __restrict__ gv = static_cast<const float*>(a.v);
  const float* __restrict__ gw = static_cast<const float*>(a.w);
  const long long g0 = eb * NP;

  // phase 0: D1D, neighbours, q, F_x, F_y in shared memory (node order)
  for (int t = threadIdx.x; t < NQ2; t += T) sD[t] = static_cast<const float*>(a.D)[t];
  for (int t = threadIdx.x; t < 6 * nloc; t += T)
    snb[t] = (int)neighbor(a.box, eb + t / 6, t % 6);
  for (int t = threadIdx.x; t < nloc * NP; t += T) {
    const float qq = to_ct<float>(qin[g0 + t]);
    sq[t] = qq;
    sfx[t] = qq * gu[g0 + t];
    sfy[t] = qq * gv[g0 + t];
  }
  __syncthreads();

  // phase 1: element-boundary flux (mod_advect3d_eq.f90:116-140)
  const float hfx = a.box.hFsf[0], hfy = a.box.hFsf[1], hfz = a.box.hFsf[2];
  for (int t = threadIdx.x; t < nloc * NFT; t += T) {
    const int le = t / NFT;
    const int r = t - le * NFT;
    const int f = r / NFP;
    const int fp = r - f * NFP;
    int nM, nP, axis, sg;
    face_nodes<NQ>(f, fp % NQ, fp / NQ, nM, nP, axis, sg);
    const long long gM = g0 + (long long)le * NP + nM;
    const long long gP = (long long)snb[6 * le + f] * NP + nP;
    const float* gvel = (axis == 0) ? gu : (axis == 1) ? gv : gw;
    const float uM = gvel[gM], uP = gvel[gP];
    const float velM = (sg > 0) ? uM : -uM;
    const float velP = (sg > 0) ? uP : -uP;
    const float qM = sq[le * NP + nM];
    const float qP = to_ct<float>(qin[gP]);
    const float alpha = 0.5f * fabsf(velP + velM);
    const float hfs = (axis == 0) ? hfx : (axis == 1) ? hfy : hfz;
    sf[le * NFT + r] = hfs * ((qP * velP - qM * velM) - alpha * (qP - qM));
  }
  __syncthreads();

  // phase 3: one thread per (i, j) column, k walking up the column
  const float Ex = a.box.Esf[0], Ey = a.box.Esf[1], Ez = a.box.Esf[2];
  const float* __restrict__ L = static_cast<const float*>(a.Lift);
  for (int c = threadIdx.x; c < nloc * NQ2; c += T) {
    const int le = c / NQ2;
    const int col = c - le * NQ2;
    const int i = col % NQ, j = col / NQ;
    float Di[NQ], Dj[NQ], Fz[NQ];
#pragma unroll
    for (int l = 0; l < NQ; l++) {
      Di[l] = sD[l * NQ + i];
      Dj[l] = sD[l * NQ + j];
    }
    const long long gc = g0 + (long long)le * NP + col;  // node (i, j, 0)
#pragma unroll
    for (int l = 0; l < NQ; l++)
      Fz[l] = sq[le * NP + col + l * NQ2] * gw[gc + (long long)l * NQ2];
    const float* fx = sfx + le * NP;
    const float* fy = sfy + le * NP;
    const float* fl = sf + le * NFT;
#pragma unroll 2
    for (int k = 0; k < NQ; k++) {
      const float dx = reg_line_sum<P, SPLIT3>(Di, fx + j * NQ + k * NQ2, 1);
      const float dy = reg_line_sum<P, SPLIT3>(Dj, fy + i + k * NQ2, NQ);
      float Dk[NQ];
#pragma unroll
      for (int l = 0; l < NQ; l++) Dk[l] = sD[l * NQ + k];
      float dz;
      {
        // same order as line_sum: sum_l D(k,l) F_z(i,j,l)
        if constexpr (!SPLIT3) {
          dz = Dk[0] * Fz[0];
#pragma unroll
          for (int l = 1; l < NQ; l++) dz = fmaf(Dk[l], Fz[l], dz);
        } else {
          constexpr int D3 = (2 * NQ + 3) / 6;
          float t1 = Dk[0] * Fz[0];
#pragma unroll
          for (int l = 1; l < D3; l++) t1 = fmaf(Dk[l], Fz[l], t1);
          float t2 = Dk[D3] * Fz[D3];
#pragma unroll
          for (int l = D3 + 1; l < 2 * D3; l++) t2 = fmaf(Dk[l], Fz[l], t2);
          float t3 = Dk[2 * D3] * Fz[2 * D3];
#pragma unroll
          for (int l = 2 * D3 + 1; l < NQ; l++) t3 = fmaf(Dk[l], Fz[l], t3);
          dz = (t1 + t2) + t3;
        }
      }
      const int n = col + k * NQ2;
      const float lf = lift_node<P>(L + n, fl, i, j, k);
      const float dq = -(((Ex * dx + Ey * dy) + Ez * dz) + lf);
      const long long g = gc + (long long)k * NQ2;
      if (a.tend_only) {
        a.q_out[g] = f32_to_f64_bits(dq);
      } else {
        // (b*dt)*dqdt in FP32, widened by bits; the state combination stays FP64
        const double inc = f32_to_f64_bits(a.cdt_hi * dq);
        double rq = fma(a.b, qin[g], inc);
        if (a.a_nonzero) rq = fma(a.a, a.q0[g], rq);
        a.q_out[g] = rq;
      }
    }
  }
}

template <int P>
struct ColCfg {
  static constexpr int NQ2 = (P + 1) * (P + 1);
  static constexpr int EPB = (256 / NQ2) > 0 ? (256 / NQ2) : 1;
  static constexpr int THREADS = ((EPB * NQ2 + 31) / 32) * 32;
};

template <int P, bool SPLIT3>
__global__ void __launch_bounds__(ColCfg<P>::THREADS) stage_col_kernel(const StageArgs a) {
  constexpr int EPB = ColCfg<P>::EPB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const long long eb = a.elem_begin + (long long)blockIdx.x * EPB;
  const long long eend = a.elem_begin + a.elem_count;
  const int nloc = (int)((eend - eb) < EPB ? (eend - eb) : EPB);
  if (nloc <= 0) return;
  stage_block_col<P, SPLIT3>(a, eb, nloc, smem_raw);
}

template <int P, bool SPLIT3>
int launch_stage_col_impl(const StageArgs& a, cudaStream_t st) {
  using C = ColCfg<P>;
  constexpr size_t smem = col_block_smem<P>(C::EPB);
  SDG_CUDA_TRY(cudaFuncSetAttribute(stage_col_kernel<P, SPLIT3>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const long long nblk = (a.elem_count + C::EPB - 1) / C::EPB;
  if (nblk <= 0) return SDG_OK;
  if (nblk > 0x7fffffffLL) return fail(SDG_ERR_INVALID_ARG, "too many elements");
  stage_col_kernel<P, SPLIT3><<<(unsigned)nblk, C::THREADS, smem, st>>>(a);
  SDG_CUDA_TRY(cudaGetLastError());
  return SDG_OK;
}

}  // namespace sdg
