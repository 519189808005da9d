// Fused RK-stage kernel with emulated FP64 arithmetic (SDG_PREC_FP64_EMU).
//
// GB300 runs FP64 at 1/64 of the FP32 rate, so this kernel keeps on the FP64
// pipe only the operations whose rounding decides the accuracy, and runs the
// long sums in double-float (sdg_df.cuh) on the FP32 pipes:
//
//   FP64:   the line bases F0 = q u_d at each line's node 0 (rounded as the
//           reference rounds flux_x = q*u), the per-line differences
//           G_d = q u_d - F0 as one FMA (exact product minus the base, rounded
//           once), the face jumps q+ - q- and V+ - V-, and the RK combine;
//   double-float: everything else.
//
// Why differences: sum_l D(i,l) F(l) cancels heavily (D annihilates
// constants), so an error of 2^-48 |F| per operand would be amplified by
// sum|D| / |derivative| (about 200 at p=7 on 32^3).  With
//   sum_l D(i,l) F(l) = sum_l D(i,l) G(l) + F(0) * R(i),  R(i) = sum_l D(i,l)
// (R taken from the FP64 operator, not from its double-float table), the
// double-float rounding only touches the small differences G, and the result
// agrees with the FP64 oracle to about 1e-14.  The upwind flux is rewritten
// the same way: qP VP - qM VM - alpha (qP - qM) = qP (VP - VM) + (qP - qM)(VM
// - alpha), with the jumps formed in FP64 (mod_advect3d_eq.f90:124-139).
//
// Layout and schedule: one block owns EPB elements and one thread one
// "line" (Nq nodes along an axis) per phase, so each loaded value feeds Nq
// outputs.  Per element, shared memory holds three planes of Np slots (one
// per axis, each laid out line-major for its axis with a pad of one slot per
// line against bank conflicts): the double-float differences G, then the
// running compensated sums (in the x plane).  Phases:
//   0  tables, neighbour elements, line bases F0 (FP64)
//   1  face fluxes g (double-float) and G = fma(q, u_d, -F0) split to
//      double-float into the planes
//   3x per x-line: sum over l for every i, plus F0 * R_x  -> running sums
//   3y per y-line: add the y sums
//   3z per z-line: add the z sums and the lift, finish the sum, RK combine.
// Escale is folded into the D tables and R; 0.5*Fscale into the lift table.
#pragma once

#include "sdg_df.cuh"
#include "sdg_stage.cuh"

namespace sdg {

template <int P>
struct EmuCfg {
  static constexpr int NQ2 = (P + 1) * (P + 1);
  static constexpr int EPB = (256 / NQ2) > 0 ? (256 / NQ2) : 1;
  static constexpr int LINES = EPB * NQ2;
  static constexpr int THREADS = ((LINES + 31) / 32) * 32;
  static constexpr int PADL = P + 2;            // slots per line (Nq + 1)
  static constexpr int PLANE = PADL * NQ2;      // slots per plane
};

// Device table layout (float2 = hi, lo):
//   D:    [3][Nq*Nq]  Es_d * D1D(i,l) at l*Nq + i, axes x, y, z
//   R:    [3][Nq]     Es_d * sum_l D1D(i,l) from the FP64 operator
//   Lift: [6*Np]      Lift_mat(n,f) * 0.5 * Fscale(f) at n + f*Np
template <int P>
constexpr size_t emu_smem_bytes() {
  using C = EmuCfg<P>;
  constexpr int NQ = P + 1, NQ2 = NQ * NQ, NFT = 6 * NQ2;
  // tables + per element: 3 planes, 3*NQ2 line bases (FP64), NFT fluxes,
  // 6 neighbour indices (padded to 8 for alignment)
  return 8 * (size_t)(3 * NQ2 + 3 * NQ) +
         (size_t)C::EPB * (8 * 3 * C::PLANE + 8 * 3 * NQ2 + 8 * NFT + 4 * 8);
}

template <int P>
__global__ void __launch_bounds__(EmuCfg<P>::THREADS) stage_emu_kernel(const StageArgs a) {
  using O = Ord<P>;
  using C = EmuCfg<P>;
  constexpr int NQ = O::NQ, NQ2 = O::NQ2, NP = O::NP, NFP = O::NFP, NFT = O::NFT,
                EPB = C::EPB, PADL = C::PADL, PLANE = C::PLANE;
  const int T = blockDim.x;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* sD = reinterpret_cast<float2*>(smem_raw);     // [3][NQ2]
  float2* sR = sD + 3 * NQ2;                            // [3][NQ]
  double* sPl = reinterpret_cast<double*>(sR + 3 * NQ); // [EPB][3][PLANE] (FP64 or float2)
  double* sF0 = sPl + EPB * 3 * PLANE;                  // [EPB][3][NQ2] line bases
  float2* sg = reinterpret_cast<float2*>(sF0 + EPB * 3 * NQ2);  // [EPB][NFT]
  int* snb = reinterpret_cast<int*>(sg + EPB * NFT);             // [EPB][8]

  const long long eb = a.elem_begin + (long long)blockIdx.x * EPB;
  const long long eend = a.elem_begin + a.elem_count;
  const int nloc = (int)((eend - eb) < EPB ? (eend - eb) : EPB);
  if (nloc <= 0) return;
  const double* __restrict__ qin = a.q_in;
  const double* __restrict__ gu = static_cast<const double*>(a.u);
  const double* __restrict__ gv = static_cast<const double*>(a.v);
  const double* __restrict__ gw = static_cast<const double*>(a.w);
  const long long g0 = eb * NP;

  // slot of node (i,j,k) in the plane of axis d (line-major for that axis)
  auto slot = [](int d, int i, int j, int k) -> int {
    return (d == 0) ? i + PADL * (j + NQ * k) : (d == 1) ? j + PADL * (i + NQ * k)
                                                         : k + PADL * (i + NQ * j);
  };

  // phase 0: tables, neighbour elements, line bases F0 = q u_d at node 0
  {
    const float2* tab = static_cast<const float2*>(a.D);
    for (int t = threadIdx.x; t < 3 * NQ2 + 3 * NQ; t += T) sD[t] = tab[t];
  }
  for (int t = threadIdx.x; t < 6 * nloc; t += T)
    snb[8 * (t / 6) + t % 6] = (int)neighbor(a.box, eb + t / 6, t % 6);
  for (int r = threadIdx.x; r < nloc * 3 * NQ2; r += T) {
    const int le = r / (3 * NQ2);
    const int rr = r - le * 3 * NQ2;
    const int d = rr / NQ2, line = rr - d * NQ2;
    const int la = line % NQ, lb = line / NQ;
    // node 0 of the line: x-line (0, j, k), y-line (i, 0, k), z-line (i, j, 0)
    const int n0 = (d == 0) ? NQ * la + NQ2 * lb : (d == 1) ? la + NQ2 * lb : la + NQ * lb;
    const long long g = g0 + (long long)le * NP + n0;
    const double* gvel = (d == 0) ? gu : (d == 1) ? gv : gw;
    sF0[r] = qin[g] * gvel[g];
  }
  __syncthreads();

  // phase 1a: upwind face fluxes g = qP (VP - VM) + (qP - qM)(VM - alpha)
  const FaceTasks<NQ> ftask(nloc);  // face-major below p = 5
  for (int t = threadIdx.x; t < nloc * NFT; t += T) {
    int le, f, fp;
    ftask.map(t, le, f, fp);
    const int ti = le * NFT + f * NFP + fp;  // element-major index of the task
    int nM, nP, axis, sgi;
    face_nodes<NQ>(f, fp % NQ, fp / NQ, nM, nP, axis, sgi);
    const long long gM = g0 + (long long)le * NP + nM;
    const long long gP = (long long)snb[8 * le + f] * NP + nP;
    const double* gvel = (axis == 0) ? gu : (axis == 1) ? gv : gw;
    const double qM = qin[gM], qP = qin[gP];
    // normal velocities +-u_axis: a sign flip, not an FP64 multiply
    const double VM = (sgi > 0) ? gvel[gM] : -gvel[gM];
    const double VP = (sgi > 0) ? gvel[gP] : -gvel[gP];
    const double jq = qP - qM, jV = VP - VM;  // FP64 jumps
    const dfl dVM = df_split(VM);
    const dfl alpha = df_scale2(df_abs(df_add(df_split(VP), dVM)), 0.5f);
    dacc A = dacc_zero();
    dacc_fma(A, df_split(qP), df_split(jV));
    dacc_fma(A, df_split(jq), df_sub(dVM, alpha));
    const dfl gf = dacc_result(A);
    sg[ti] = make_float2(gf.hi, gf.lo);
  }
  // phase 1b: G = q u_d - F0 (one FMA), split to double-float into the planes
  for (int t = threadIdx.x; t < nloc * NP; t += T) {
    const int le = t / NP;
    const int n = t - le * NP;
    const int i = n % NQ, j = (n / NQ) % NQ, k = n / NQ2;
    float2* pl = reinterpret_cast<float2*>(sPl + le * 3 * PLANE);
    const double* f0 = sF0 + le * 3 * NQ2;
    const double qq = qin[g0 + t];
    const dfl Gx = df_split(fma(qq, gu[g0 + t], -f0[0 * NQ2 + j + NQ * k]));
    const dfl Gy = df_split(fma(qq, gv[g0 + t], -f0[1 * NQ2 + i + NQ * k]));
    const dfl Gz = df_split(fma(qq, gw[g0 + t], -f0[2 * NQ2 + i + NQ * j]));
    pl[0 * PLANE + slot(0, i, j, k)] = make_float2(Gx.hi, Gx.lo);
    pl[1 * PLANE + slot(1, i, j, k)] = make_float2(Gy.hi, Gy.lo);
    pl[2 * PLANE + slot(2, i, j, k)] = make_float2(Gz.hi, Gz.lo);
  }
  __syncthreads();

  // phase 3: one thread per line, Nq outputs per line
  const int r = threadIdx.x;
  const bool has_line = r < nloc * NQ2;
  const int le = has_line ? r / NQ2 : 0;
  const int line = r - le * NQ2;
  const int la = line % NQ, lb = line / NQ;
  float2* pl2 = reinterpret_cast<float2*>(sPl + le * 3 * PLANE);
  const double* f0 = sF0 + le * 3 * NQ2;

  // 3x: line (j, k) = (la, lb); running sums go to the x plane in place
  if (has_line) {
    float2 Gl[NQ];
#pragma unroll
    for (int l = 0; l < NQ; l++) Gl[l] = pl2[PADL * line + l];
    const dfl base = df_split(f0[0 * NQ2 + line]);
#pragma unroll
    for (int i = 0; i < NQ; i++) {
      dacc A = dacc_zero();
#pragma unroll
      for (int l = 0; l < NQ; l++) {
        const float2 dd = sD[0 * NQ2 + l * NQ + i];
        dacc_fma(A, df_make(dd.x, dd.y), df_make(Gl[l].x, Gl[l].y));
      }
      const float2 rr = sR[0 * NQ + i];
      dacc_fma(A, df_make(rr.x, rr.y), base);
      pl2[PADL * line + i] = make_float2(A.s, A.c);
    }
  }
  __syncthreads();

  // 3y: line (i, k) = (la, lb)
  if (has_line) {
    const int i = la, k = lb;
    float2 Gl[NQ];
#pragma unroll
    for (int l = 0; l < NQ; l++) Gl[l] = pl2[1 * PLANE + PADL * line + l];
    const dfl base = df_split(f0[1 * NQ2 + line]);
#pragma unroll
    for (int j = 0; j < NQ; j++) {
      const int s = i + PADL * (j + NQ * k);
      const float2 acc = pl2[s];
      dacc A;
      A.s = acc.x;
      A.c = acc.y;
#pragma unroll
      for (int l = 0; l < NQ; l++) {
        const float2 dd = sD[1 * NQ2 + l * NQ + j];
        dacc_fma(A, df_make(dd.x, dd.y), df_make(Gl[l].x, Gl[l].y));
      }
      const float2 rr = sR[1 * NQ + j];
      dacc_fma(A, df_make(rr.x, rr.y), base);
      pl2[s] = make_float2(A.s, A.c);
    }
  }
  __syncthreads();

  // 3z: line (i, j) = (la, lb); lift, finish, RK combine, store
  if (has_line) {
    const int i = la, j = lb;
    float2 Gl[NQ];
#pragma unroll
    for (int l = 0; l < NQ; l++) Gl[l] = pl2[2 * PLANE + PADL * line + l];
    const dfl base = df_split(f0[2 * NQ2 + line]);
    const float2* __restrict__ Lt = static_cast<const float2*>(a.Lift);
    const float2* gl = sg + le * NFT;
    const dfl c_dt = df_make(a.cdt_hi, a.cdt_lo);
    with_rk_kind(rk_kind(a), [&](auto rkc) {
      constexpr int RK = decltype(rkc)::value;
#pragma unroll 1
      for (int k = 0; k < NQ; k++) {
        const int s = i + PADL * (j + NQ * k);
        const float2 acc = pl2[s];
        dacc A;
        A.s = acc.x;
        A.c = acc.y;
#pragma unroll
        for (int l = 0; l < NQ; l++) {
          const float2 dd = sD[2 * NQ2 + l * NQ + k];
          dacc_fma(A, df_make(dd.x, dd.y), df_make(Gl[l].x, Gl[l].y));
        }
        const float2 rr = sR[2 * NQ + k];
        dacc_fma(A, df_make(rr.x, rr.y), base);
        const int n = i + j * NQ + k * NQ2;
        const int fidx[6] = {i + k * NQ, NFP + j + k * NQ, 2 * NFP + i + k * NQ,
                             3 * NFP + j + k * NQ, 4 * NFP + i + j * NQ, 5 * NFP + i + j * NQ};
#pragma unroll
        for (int f = 0; f < 6; f++) {
          const float2 L = __ldg(Lt + n + f * NP);
          const float2 gg = gl[fidx[f]];
          dacc_fma(A, df_make(L.x, L.y), df_make(gg.x, gg.y));
        }
        const dfl dq = df_neg(dacc_result(A));
        const long long g = (eb + le) * NP + n;
        if constexpr (RK == kRkTend) {
          a.q_out[g] = f32_to_f64_bits(dq.hi) + f32_to_f64_bits(dq.lo);
        } else {
          const dfl inc = df_mul(c_dt, dq);  // (b*dt)*dqdt
          const double ih = f32_to_f64_bits(inc.hi), il = f32_to_f64_bits(inc.lo);
          const double qv = qin[g];
          if constexpr (RK == kRkFirst)
            a.q_out[g] = (qv + ih) + il;
          else
            a.q_out[g] = fma(a.a, a.q0[g], fma(a.b, qv, ih) + il);
        }
      }
    });
  }
}

template <int P>
int launch_stage_emu_impl(const StageArgs& a, cudaStream_t st) {
  using C = EmuCfg<P>;
  constexpr size_t smem = emu_smem_bytes<P>();
  SDG_TRY(set_kernel_smem((const void*)stage_emu_kernel<P>, (int)smem, false));
  const long long nblk = (a.elem_count + C::EPB - 1) / C::EPB;
  if (nblk <= 0) return SDG_OK;
  if (nblk > 0x7fffffffLL) return fail(SDG_ERR_INVALID_ARG, "too many elements");
  stage_emu_kernel<P><<<(unsigned)nblk, C::THREADS, smem, st>>>(a);
  SDG_CUDA_TRY(cudaGetLastError());
  return SDG_OK;
}

}  // namespace sdg
