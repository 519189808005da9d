// Fused SSP-RK3 stage for meshes given as the reference's arrays: the time
// loop of main.f90:51-80 (q0 = q; per stage update_halo(q),
// advect3d_eq_cal_tend (mod_advect3d_eq.f90:41-85), RK update) in one launch
// per stage, with the even-odd line sums of the fused structured stage.
//
// What the caller's arrays decide, and how they are honoured:
//   * VMapM / VMapP (1-based flat DOF ids, halo slots for periodic
//     neighbours): resolved once per call through halo_src_map to the owned
//     node each one reads (step_face_kernel), so the stages gather q from
//     the owned part of the previous stage's state -- the value update_halo
//     would have copied into the slot -- and need no halo copy of their own.
//     The velocity gathers use VMapM / VMapP as given (the caller's u, v, w
//     halos), as cal_elembnd_flux does;
//   * normal_fn and Fscale: the face flux
//       0.5 Fs ((qP VelP - qM VelM) - alpha (qP - qM)),  Vel = u.n,
//       alpha = 0.5 |VelP + VelM|  (mod_advect3d_eq.f90:116-140)
//     is formed as qP tP - qM tM with tP = 0.5 Fs (VelP - alpha) and
//     tM = 0.5 Fs (VelM - alpha).  tP and tM depend only on the velocity and
//     the geometry, which every stage of the loop shares (main.f90:58-67
//     passes the same u, v, w each time and never changes them), so
//     step_face_kernel forms them once per call and every stage reads them;
//   * Escale (per node, per direction): applied to each direction's
//     derivative sum before the lift is added, as cal_dqdt does
//     (mod_advect3d_eq.f90:185-198).  Where an element's Escale is one value
//     per direction (mesh_setup's affine elements, mod_mesh.f90:147-149;
//     step_escale_kernel checks every node once per call) the value is
//     folded into that element's copy of the derivative tables instead, and
//     its lines run the structured stage's body (eo_line); elements with
//     Escale varying node by node keep the per-node form (eo_line_esc).
// The summation order is the even-odd one of dqdt_eo_kernel: neither
// GENERAL's nor OPT1's, equal to both to rounding.
#pragma once

#include "sdg_stage.cuh"
#include "sdg_stage_eo.cuh"

namespace sdg {

struct StepRefArgs {
  const double* q_in;   // stage input state, owned part (Np*Ne)
  const double* q0;     // step-start state (stages 2 and 3)
  double* q_out;        // stage result (Np*Ne); may be q0 in the third stage
  const double* u;      // caller's velocity with halos (Np*NeA)
  const double* v;
  const double* w;
  const double* tab;    // 3 x TE unscaled even-odd tables (step_tables_kernel)
  const int2* res;      // per face node: the 0-based owned nodes qM and qP come
                        //   from (-1: a map entry was out of range)
  const double2* fc;    // per face node: the velocity factors (tP, tM)
  const double* Escale;
  const double4* esu;   // per element: (Es_x, Es_y, Es_z, 1) when its Escale is
                        //   one value per direction, (.., 0) otherwise
  int Ne;
  double a, b, c;       // q_out = a q0 + b q_in + c S, c = -b dt, S = -dqdt
                        // (the tables are scaled by c)
  int rk;               // kRkFirst or kRkGeneral
};

template <int P>
struct StepRefCfg {
  static constexpr int THREADS = 256;
  static constexpr int EPB = (256 / Ord<P>::NQ2) > 0 ? 256 / Ord<P>::NQ2 : 1;
};

template <int P>
constexpr size_t step_ref_smem_bytes() {
  using O = Ord<P>;
  return sizeof(double) * (size_t)(3 * EoShape<P>::TE +
                                   StepRefCfg<P>::EPB * (O::NP + O::NFT + 3 * EoShape<P>::TE));
}

// The three directions' unscaled even-odd tables from D1D and Lift_mat (the
// lift column of a face from its tangential node (0, 0)), one block; it
// checks the symmetries the factorisation needs -- D1D centro-antisymmetric,
// D1D_tr its transpose, each face's lift constant over the tangential nodes,
// the + face's column the mirror of the - face's, all to 1e-13 of the largest
// entry -- and sets *err = 2 when one fails.
template <int P>
__global__ void __launch_bounds__(256) step_tables_kernel(const double* __restrict__ D,
                                                          const double* __restrict__ Dt,
                                                          const double* __restrict__ L,
                                                          double* tab, int* err) {
  using O = Ord<P>;
  using Sh = EoShape<P>;
  constexpr int NQ = O::NQ, NQ2 = O::NQ2, NP = O::NP, TE = Sh::TE, N = Sh::N, H = Sh::H;
  __shared__ unsigned long long smax[2];
  auto Dv = [&](int i, int l) { return D[i + l * N]; };  // D1D(i,l), column-major
  auto Ds = [&](int i, int l) { return 0.5 * (Dv(i, l) - Dv(N - 1 - i, N - 1 - l)); };
  auto node = [](int ax, int m, int t1, int t2) {
    return (ax == 0) ? m + NQ * t1 + NQ2 * t2 : (ax == 1) ? t1 + NQ * m + NQ2 * t2
                                                           : t1 + NQ * t2 + NQ2 * m;
  };
  auto col = [&](int ax, int side, int m) {
    const int f = (ax == 0) ? (side ? 1 : 3) : (ax == 1) ? (side ? 2 : 0) : (side ? 5 : 4);
    return L[node(ax, m, 0, 0) + (long long)f * NP];
  };
  auto lam = [&](int ax, int m) { return 0.5 * (col(ax, 0, m) + col(ax, 1, N - 1 - m)); };
  for (int t = threadIdx.x; t < 3 * TE; t += blockDim.x) {
    const int ax = t / TE, w = t - ax * TE;
    double v;
    if (w < Sh::OFF_O) {
      const int i = w / H, l = w - i * H;
      v = 0.5 * (Ds(i, l) + Ds(i, N - 1 - l));
    } else if (w < Sh::OFF_DM) {
      const int i = (w - Sh::OFF_O) / H, l = (w - Sh::OFF_O) - i * H;
      v = 0.5 * (Ds(i, l) - Ds(i, N - 1 - l));
    } else if (w < Sh::OFF_A) {
      v = Ds(w - Sh::OFF_DM, H);
    } else if (w < Sh::OFF_B) {
      const int i = w - Sh::OFF_A;
      v = 0.5 * (lam(ax, i) + lam(ax, N - 1 - i));
    } else {
      const int i = w - Sh::OFF_B;
      v = 0.5 * (lam(ax, i) - lam(ax, N - 1 - i));
    }
    tab[t] = v;
  }
  if (threadIdx.x == 0) smax[0] = smax[1] = 0ull;
  __syncthreads();
  unsigned long long mD = 0, mL = 0;
  for (int t = threadIdx.x; t < NQ2; t += blockDim.x)
    mD = max(mD, (unsigned long long)__double_as_longlong(fabs(D[t])));
  for (int t = threadIdx.x; t < 6 * NP; t += blockDim.x)
    mL = max(mL, (unsigned long long)__double_as_longlong(fabs(L[t])));
  atomicMax(&smax[0], mD);
  atomicMax(&smax[1], mL);
  __syncthreads();
  const double tD = 1e-13 * __longlong_as_double((long long)smax[0]);
  const double tL = 1e-13 * __longlong_as_double((long long)smax[1]);
  bool bad = false;
  for (int t = threadIdx.x; t < NQ2; t += blockDim.x) {
    const int i = t % N, l = t / N;
    bad |= fabs(Dv(i, l) + Dv(N - 1 - i, N - 1 - l)) > tD;
    bad |= fabs(Dt[l + i * N] - Dv(i, l)) > tD;
  }
  for (int t = threadIdx.x; t < 6 * NP; t += blockDim.x) {
    const int f = t / NP, n = t - f * NP;
    const int ax = (f == 1 || f == 3) ? 0 : (f == 0 || f == 2) ? 1 : 2;
    const int side = (f == 1 || f == 2 || f == 5) ? 1 : 0;
    const int c[3] = {n % NQ, (n / NQ) % NQ, n / NQ2};
    bad |= fabs(L[t] - col(ax, side, c[ax])) > tL;
    if (n < N && ax == 0 && side == 0)
      for (int x = 0; x < 3; x++) bad |= fabs(col(x, 0, n) - col(x, 1, N - 1 - n)) > tL;
  }
  if (bad) atomicExch(err, 2);
}

// One line in pair form with the caller's per-node Escale: row holds S(l) at
// l and Δ(l) at N-1-l (l < N/2) and F(mid) for an odd N; T the direction's
// tables scaled by the stage factor c; gm / gp the line's face fluxes; Es(m)
// the node's Escale.  emit(m, r) receives r = Es(m) (D F)(m) + lift(m), both
// times c.  Per output pair: the even and odd sums, e + o and o - e, one
// product B gd shared by the two lifts (A gs +- B gd) and two FMAs with
// Escale -- seven FP64 operations beside the sums.
template <int P, typename EsAt, typename Emit>
__device__ __forceinline__ void eo_line_esc(const double* row, const double* __restrict__ T,
                                            double gm, double gp, EsAt&& Es, Emit&& emit) {
  using Sh = EoShape<P>;
  constexpr int N = Sh::N, H = Sh::H;
  double sv[H], dv[H];
#pragma unroll
  for (int l = 0; l < H; l++) {
    sv[l] = row[l];
    dv[l] = row[N - 1 - l];
  }
  double fm = 0.0;
  if constexpr (Sh::ODD != 0) fm = row[H];
  const double gs = gm + gp, gd = gm - gp;
  constexpr int kRowUnroll = (N <= 5) ? H : 1;
#pragma unroll kRowUnroll
  for (int i = 0; i < H; i++) {
    double e = T[Sh::OFF_E + i * H] * sv[0];
#pragma unroll
    for (int l = 1; l < H; l++) e = fma(T[Sh::OFF_E + i * H + l], sv[l], e);
    if constexpr (Sh::ODD != 0) e = fma(T[Sh::OFF_DM + i], fm, e);
    double o = T[Sh::OFF_O + i * H] * dv[0];
#pragma unroll
    for (int l = 1; l < H; l++) o = fma(T[Sh::OFF_O + i * H + l], dv[l], o);
    const double bg = T[Sh::OFF_B + i] * gd, ag = T[Sh::OFF_A + i];
    emit(i, fma(Es(i), e + o, fma(ag, gs, bg)));
    emit(N - 1 - i, fma(Es(N - 1 - i), o - e, fma(ag, gs, -bg)));
  }
  if constexpr (Sh::ODD != 0) {
    double o = T[Sh::OFF_O + H * H] * dv[0];
#pragma unroll
    for (int l = 1; l < H; l++) o = fma(T[Sh::OFF_O + H * H + l], dv[l], o);
    emit(H, fma(Es(H), o, T[Sh::OFF_A + H] * gs));
  }
}

// One stage over elements [blockIdx.x*EPB, ...): the face fluxes from the
// per-call face data, the even-odd line sums with per-node Escale, the lift
// and the RK update.  One thread per line in the line phases.
template <int P, int RK>
__global__ void __launch_bounds__(StepRefCfg<P>::THREADS, 4) step_ref_kernel(const StepRefArgs a) {
  using O = Ord<P>;
  using Sh = EoShape<P>;
  constexpr int NQ = O::NQ, NQ2 = O::NQ2, NP = O::NP, NFP = O::NFP, NFT = O::NFT,
                EPB = StepRefCfg<P>::EPB, T = StepRefCfg<P>::THREADS, TE = Sh::TE,
                H = Sh::H, HR = Sh::HR;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* sT = reinterpret_cast<double*>(smem_raw);  // [3][TE]
  double* sA = sT + 3 * TE;                          // [EPB][NP]: x pairs, then sums
  double* sf = sA + EPB * NP;                        // [EPB][NFT] face fluxes
  double* sTe = sf + EPB * NFT;                      // [EPB][3][TE] per element
  const long long eb = (long long)blockIdx.x * EPB;
  const int nloc = (int)min((long long)EPB, (long long)a.Ne - eb);
  if (nloc <= 0) return;
  // the tables times the stage factor c = -b dt: the line results are then
  // the stage's increments, and the RK update needs no multiply of its own;
  // an element with one Escale per direction gets its own copy with the
  // derivative parts also times Es_d
  for (int t = threadIdx.x; t < 3 * TE; t += T) sT[t] = a.tab[t] * a.c;
  for (int t = threadIdx.x; t < nloc * 3 * TE; t += T) {
    const int le = t / (3 * TE), w3 = t - le * 3 * TE, dir = w3 / TE, w = w3 - dir * TE;
    const double4 es = a.esu[eb + le];
    const double sd = (dir == 0) ? es.x : (dir == 1) ? es.y : es.z;
    sTe[t] = (w < Sh::OFF_A) ? a.tab[w3] * (a.c * sd) : a.tab[w3] * a.c;
  }
  const long long g0 = eb * NP;
  const double* __restrict__ q = a.q_in;
  const double* __restrict__ gu = a.u;
  // x pair values: one task per (element, x line, c < ceil(N/2))
  for (int t = threadIdx.x; t < nloc * NQ2 * HR; t += T) {
    const int le = t / (NQ2 * HR), w = t - le * NQ2 * HR;
    const int r = w / HR, c = w - r * HR;
    const long long g = g0 + (long long)le * NP + (long long)r * NQ;
    double* row = sA + le * NP + r * NQ;
    if (c < H) {
      const double q1 = q[g + c], u1 = gu[g + c];
      const double p2 = q[g + NQ - 1 - c] * gu[g + NQ - 1 - c];
      row[c] = fma(q1, u1, p2);
      row[NQ - 1 - c] = fma(q1, u1, -p2);
    } else {
      row[c] = q[g + c] * gu[g + c];
    }
  }
  // face fluxes qP tP - qM tM
  for (int t = threadIdx.x; t < nloc * NFT; t += T) {
    const long long m = eb * NFT + t;
    const int2 rr = a.res[m];
    const double2 fc = a.fc[m];
    sf[t] = (rr.x >= 0) ? fma(q[rr.y], fc.x, -(q[rr.x] * fc.y)) : 0.0;
  }
  __syncthreads();
  const long long NpNe = (long long)NP * a.Ne;
  const double* __restrict__ Es = a.Escale;
  const int r = threadIdx.x % NQ2, le = threadIdx.x / NQ2;
  const bool has_line = threadIdx.x < nloc * NQ2;
  const double* fl = sf + le * NFT + r;
  // one Escale per direction for this line's element: the folded tables
  const bool uni = has_line && a.esu[eb + le].w != 0.0;
  const double* Te = sTe + le * 3 * TE;
  // x lines: faces -x (3) and +x (1); Escale_x D F + lift over the pair values
  if (has_line) {
    double* row = sA + le * NP + r * NQ;
    const long long g = g0 + (long long)le * NP + (long long)r * NQ;
    auto emit = [&](int m, double r) { row[m] = r; };
    if (uni)
      eo_line<P, 1, 1, true>(row, Te, fl[3 * NFP], fl[1 * NFP], 0, emit);
    else
      eo_line_esc<P>(row, sT, fl[3 * NFP], fl[1 * NFP], [&](int m) { return Es[g + m]; }, emit);
  }
  __syncthreads();
  // y lines: faces -y (0) and +y (2); added into the sums
  if (has_line) {
    const int off = le * NP + (r % NQ) + (r / NQ) * NQ2;
    double row[NQ];
    eo_pairs_f64<P>(q, a.v, g0 + off, NQ, row);
    auto emit = [&](int m, double r) { sA[off + m * NQ] += r; };
    if (uni)
      eo_line<P, 1, 1, true>(row, Te + TE, fl[0], fl[2 * NFP], 0, emit);
    else
      eo_line_esc<P>(row, sT + TE, fl[0], fl[2 * NFP],
                     [&](int m) { return Es[g0 + off + m * NQ + NpNe]; }, emit);
  }
  __syncthreads();
  // z lines: faces -z (4) and +z (5); finish the node and the RK update
  if (has_line) {
    const int off = le * NP + r;
    double row[NQ];
    eo_pairs_f64<P>(q, a.w, g0 + off, NQ2, row);
    double* __restrict__ qout = a.q_out;
    const double* q0 = a.q0;
    const double ra = a.a, rb = a.b;
    auto emit = [&](int m, double r) {
      const int n = off + m * NQ2;
      const long long g = g0 + n;
      // q0 is read before q_out is written at the same node, by this thread
      // only, so the third stage may write the result over q0
      qout[g] = rk_combine<RK>(sA[n] + r, q[g], RK == kRkGeneral ? q0[g] : 0.0, ra, rb);
    };
    if (uni)
      eo_line<P, 1, 1, true>(row, Te + 2 * TE, fl[4 * NFP], fl[5 * NFP], 0, emit);
    else
      eo_line_esc<P>(row, sT + 2 * TE, fl[4 * NFP], fl[5 * NFP],
                     [&](int m) { return Es[g0 + off + m * NQ2 + 2 * NpNe]; }, emit);
  }
}

template <int P>
int launch_step_ref_impl(const StepRefArgs& a, cudaStream_t st) {
  constexpr size_t smem = step_ref_smem_bytes<P>();
  const long long nblk = ((long long)a.Ne + StepRefCfg<P>::EPB - 1) / StepRefCfg<P>::EPB;
  if (nblk == 0) return SDG_OK;
  if (a.rk == kRkFirst) {
    SDG_TRY(set_kernel_smem((const void*)step_ref_kernel<P, kRkFirst>, (int)smem, false));
    step_ref_kernel<P, kRkFirst><<<(unsigned)nblk, StepRefCfg<P>::THREADS, smem, st>>>(a);
  } else {
    SDG_TRY(set_kernel_smem((const void*)step_ref_kernel<P, kRkGeneral>, (int)smem, false));
    step_ref_kernel<P, kRkGeneral><<<(unsigned)nblk, StepRefCfg<P>::THREADS, smem, st>>>(a);
  }
  SDG_CUDA_TRY(cudaGetLastError());
  return SDG_OK;
}

}  // namespace sdg
