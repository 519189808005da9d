// Emulated-FP64 stage with the even-odd factorisation (SDG_PREC_FP64_EMU with
// SDG_OPT_EVENODD): the accuracy scheme of stage_emu_kernel (FP64
// differences, double-float sums) on the pair structure of stage_eo_block.
//
// Per line of an axis d, with the line base F0 = q u_d at the line's node 0
// and the differences G(l) = q u_d - F0 formed by one FP64 FMA (exact product
// minus the base, rounded once) and split to double-float, the pair values
//     S(l) = G(l) + G(N-1-l),   Δ(l) = G(l) - G(N-1-l)      (l < N/2)
// are double-float sums (TwoSum, no FP64 instruction: the differences are of
// the size of the line's variation, so S and Δ keep 2^-48 of it), and
//     e_i = Σ_l E(i,l) S(l) + R(i) F0 [+ D(i,mid) G(mid)] + B(i) gd,
//     o_i = Σ_l O(i,l) Δ(l) + A(i) gs,
//     out(i) = e_i + o_i,  out(N-1-i) = o_i - e_i,
// with compensated (Dot2) double-float sums.  R is the row sum of the
// symmetrised FP64 operator, antisymmetric in i, so the base term joins e.
// The tables carry -Escale (D part) and -0.5*Fscale (lift part), so the three
// line results sum to dqdt; the RK update runs in FP64 as in stage_emu_kernel.
//
// A line costs about N/2 + 2 compensated products per output instead of
// N + 1 (plus the lift, which joins the same pairs).
//
// Shared memory per element: one plane of double-float values, line-major for
// the x axis with a pad slot per line (first the x pair values, then the
// running compensated sums of the nodes), the x line bases, the face fluxes
// and the neighbour indices.  The y and z pair values are formed by the line
// threads of those phases from q and v / w in global memory (cached), which
// keeps the footprint at a third and lets four blocks share an SM.
#pragma once

#include "sdg_df.cuh"
#include "sdg_stage.cuh"
#include "sdg_stage_eo.cuh"

namespace sdg {

// Lines a block aims at: 256, or 128 at p = 7, where twice as many half-size
// blocks (the same warps an SM) measured 1.05x on GB300 (0.89-0.99x at p = 5,
// 9 and 10), and at p <= 4 with twelve blocks an SM (1.04-1.06x: 32.0
// against 30.2 GDOF-updates/s at p = 1, 44.6 against 42.4 at p = 3).
template <int P>
struct EmuEoCfg {
  static constexpr int NQ2 = (P + 1) * (P + 1);
  static constexpr int AIM = (P == 7 || P <= 4) ? 128 : 256;
  static constexpr int EPB = (AIM / NQ2) > 0 ? (AIM / NQ2) : 1;
  static constexpr int LINES = EPB * NQ2;
  static constexpr int THREADS = ((LINES + 31) / 32) * 32;
  static constexpr int PADL = P + 2;        // slots per line (N + 1)
  static constexpr int PLANE = PADL * NQ2;  // slots per plane
  static constexpr int TE = EoShape<P>::TE + EoShape<P>::H;  // + R(i), i < H
  static constexpr int OFF_R = EoShape<P>::TE;
};

// Device table (float2 = hi, lo), per axis x, y, z: E, O, D(i,mid), A, B as in
// EoShape (D parts times -Es_d, lift parts times -0.5*Fs_d), then R(i) times
// -Es_d for i < N/2.
template <int P>
constexpr size_t emu_eo_smem_bytes() {
  using C = EmuEoCfg<P>;
  constexpr int NQ = P + 1, NQ2 = NQ * NQ, NFT = 6 * NQ2;
  return 8 * (size_t)(3 * C::TE) +
         (size_t)C::EPB * (8 * C::PLANE + 8 * NQ2 + 8 * NFT + 4 * 8);
}

// Pair values of one line from global memory: F0 = q u at the line's node 0,
// G = q u - F0 by one FMA, split, S and Δ in double-float; written to
// row[0..N).
template <int P>
__device__ __forceinline__ void emu_eo_pairs(const double* __restrict__ q,
                                             const double* __restrict__ vel, long long g0,
                                             int stride, float2* row, double& f0) {
  using Sh = EoShape<P>;
  constexpr int N = Sh::N, H = Sh::H;
  f0 = q[g0] * vel[g0];
#pragma unroll
  for (int c = 0; c < H; c++) {
    const long long a = g0 + (long long)c * stride, b = g0 + (long long)(N - 1 - c) * stride;
    const dfl g1 = df_split(fma(q[a], vel[a], -f0));
    const dfl g2 = df_split(fma(q[b], vel[b], -f0));
    const dfl S = df_add(g1, g2), D = df_sub(g1, g2);
    row[c] = make_float2(S.hi, S.lo);
    row[N - 1 - c] = make_float2(D.hi, D.lo);
  }
  if constexpr (Sh::ODD != 0) {
    const long long a = g0 + (long long)H * stride;
    const dfl M = df_split(fma(q[a], vel[a], -f0));
    row[H] = make_float2(M.hi, M.lo);
  }
}

__device__ __forceinline__ dacc dacc_of(dfl a) {
  dacc r;
  r.s = a.hi;
  r.c = a.lo;
  return r;
}

// o + e (MINUS = false) or o - e (MINUS = true) of two compensated sums.
template <bool MINUS>
__device__ __forceinline__ dacc dacc_combine(const dacc& o, const dacc& e) {
  const float es = MINUS ? -e.s : e.s, ec = MINUS ? -e.c : e.c;
  const dfl t = two_sum(o.s, es);
  dacc r;
  r.s = t.hi;
  r.c = DFA(DFA(o.c, ec), t.lo);
  return r;
}

// acc += x
__device__ __forceinline__ void dacc_accum(dacc& acc, const dacc& x) {
  const dfl t = two_sum(acc.s, x.s);
  acc.s = t.hi;
  acc.c = DFA(acc.c, DFA(x.c, t.lo));
}

__device__ __forceinline__ dfl f2_df(float2 v) { return df_make(v.x, v.y); }

// One line of axis tables T: pair values (S at l, Δ at N-1-l, G(mid) at H) in
// the row `row`, base b0, face fluxes gm / gp.  emit(m, sum) receives the
// compensated result for position m, after all reads of the row.
template <int P, typename Emit>
__device__ __forceinline__ void emu_eo_line(const float2* row, const float2* __restrict__ T,
                                            dfl b0, dfl gm, dfl gp, Emit&& emit) {
  using Sh = EoShape<P>;
  using C = EmuEoCfg<P>;
  constexpr int N = Sh::N, H = Sh::H;
  dfl s[H], d[H];
#pragma unroll
  for (int l = 0; l < H; l++) {
    s[l] = f2_df(row[l]);
    d[l] = f2_df(row[N - 1 - l]);
  }
  dfl gmid = df_make(0.f, 0.f);
  if constexpr (Sh::ODD != 0) gmid = f2_df(row[H]);
  const dfl gs = df_add(gm, gp), gd = df_sub(gm, gp);
#pragma unroll 1
  for (int i = 0; i < H; i++) {
    dacc e = dacc_zero();
#pragma unroll
    for (int l = 0; l < H; l++) dacc_fma(e, f2_df(T[Sh::OFF_E + i * H + l]), s[l]);
    dacc_fma(e, f2_df(T[C::OFF_R + i]), b0);
    if constexpr (Sh::ODD != 0) dacc_fma(e, f2_df(T[Sh::OFF_DM + i]), gmid);
    dacc_fma(e, f2_df(T[Sh::OFF_B + i]), gd);
    dacc o = dacc_zero();
#pragma unroll
    for (int l = 0; l < H; l++) dacc_fma(o, f2_df(T[Sh::OFF_O + i * H + l]), d[l]);
    dacc_fma(o, f2_df(T[Sh::OFF_A + i]), gs);
    emit(i, dacc_combine<false>(o, e));
    emit(N - 1 - i, dacc_combine<true>(o, e));
  }
  if constexpr (Sh::ODD != 0) {
    dacc o = dacc_zero();
#pragma unroll
    for (int l = 0; l < H; l++) dacc_fma(o, f2_df(T[Sh::OFF_O + H * H + l]), d[l]);
    dacc_fma(o, f2_df(T[Sh::OFF_A + H]), gs);
    emit(H, o);
  }
}

// Resident blocks of about 256 threads an SM the registers are capped for
// (twice as many of 128 at p <= 4 and p = 7).  The body waits on both the FP64 pipe
// and instruction issue, and more warps overlap the two: measured on GB300,
// six blocks (40 registers) up to p = 6 and five (48 registers, no spills) up
// to p = 12 run 1.07-1.14x four blocks; above p = 12 the caps spill and four
// blocks are faster.
template <int P>
__host__ __device__ constexpr int emu_eo_min_blocks() {
  return P <= 4 ? 12 : P <= 6 ? 6 : P == 7 ? 10 : (P <= 12 ? 5 : 4);
}

template <int P>
__global__ void __launch_bounds__(EmuEoCfg<P>::THREADS, emu_eo_min_blocks<P>())
    stage_emu_eo_kernel(const StageArgs a) {
  using O = Ord<P>;
  using Sh = EoShape<P>;
  using C = EmuEoCfg<P>;
  constexpr int NQ = O::NQ, NQ2 = O::NQ2, NP = O::NP, NFP = O::NFP, NFT = O::NFT,
                EPB = C::EPB, PADL = C::PADL, PLANE = C::PLANE, TE = C::TE, H = Sh::H,
                HR = Sh::HR;
  const int T = blockDim.x;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* sT = reinterpret_cast<float2*>(smem_raw);            // [3][TE]
  float2* sPl = sT + 3 * TE;                                   // [EPB][PLANE]
  double* sF0 = reinterpret_cast<double*>(sPl + EPB * PLANE);  // [EPB][NQ2], x lines
  float2* sg = reinterpret_cast<float2*>(sF0 + EPB * NQ2);     // [EPB][NFT]
  int* snb = reinterpret_cast<int*>(sg + EPB * NFT);           // [EPB][8]

  const long long eb = a.elem_begin + (long long)blockIdx.x * EPB;
  const long long eend = a.elem_begin + a.elem_count;
  const int nloc = (int)((eend - eb) < EPB ? (eend - eb) : EPB);
  if (nloc <= 0) return;
  const double* __restrict__ qin = a.q_in;
  const double* __restrict__ gu = static_cast<const double*>(a.u);
  const double* __restrict__ gv = static_cast<const double*>(a.v);
  const double* __restrict__ gw = static_cast<const double*>(a.w);
  const long long g0 = eb * NP;

  // node of line r of axis d at position c along the axis
  auto line_node = [](int d, int r, int c) -> int {
    return (d == 0) ? c + NQ * r : (d == 1) ? (r % NQ) + NQ * c + NQ2 * (r / NQ) : r + NQ2 * c;
  };

  // phase 0: tables, neighbour elements, line bases F0 = q u_d at node 0
  {
    const float2* tab = static_cast<const float2*>(a.D);
    for (int t = threadIdx.x; t < 3 * TE; t += T) sT[t] = tab[t];
  }
  for (int t = threadIdx.x; t < 6 * nloc; t += T)
    snb[8 * (t / 6) + t % 6] = (int)neighbor(a.box, eb + t / 6, t % 6);
  for (int t = threadIdx.x; t < nloc * NQ2; t += T) {
    const int le = t / NQ2, r = t - le * NQ2;
    const long long g = g0 + (long long)le * NP + line_node(0, r, 0);
    sF0[t] = qin[g] * gu[g];
  }
  __syncthreads();

  // phase 1a: face fluxes g = qP (VP - alpha) - qM (VM - alpha), alpha =
  // |VP + VM| / 2, formed in FP64 as the FP64 stage forms them (five
  // operations: F = qP (2 VelP - 2 alpha) - qM (2 VelM - 2 alpha) with the
  // normal sign through the constant +-2) and split once, g = F / 2 exactly.
  // Five FP64 operations a face node cost less than the two FP64 jumps, five
  // splits and two compensated products of the double-float form: that form
  // issued about a fifth of the kernel's instructions.  The velocity factors
  // tP and tM come from fc_in when an earlier stage of the same solver call
  // stored them.
  const double2* __restrict__ fcin = reinterpret_cast<const double2*>(a.fc_in);
  double2* __restrict__ fcout = reinterpret_cast<double2*>(a.fc_out);
  const FaceTasks<NQ> ftask(nloc);  // face-major below p = 5
  for (int t = threadIdx.x; t < nloc * NFT; t += T) {
    int le, f, fp;
    ftask.map(t, le, f, fp);
    const int ti = le * NFT + f * NFP + fp;  // element-major index of the task
    int nM, nP, axis, sgi;
    face_nodes<NQ>(f, fp % NQ, fp / NQ, nM, nP, axis, sgi);
    const long long gM = g0 + (long long)le * NP + nM;
    const long long gP = (long long)snb[8 * le + f] * NP + nP;
    const double qM = qin[gM], qP = qin[gP];
    double tP, tM;
    if (fcin != nullptr) {
      const double2 c = fcin[eb * NFT + ti];
      tP = c.x;
      tM = c.y;
    } else {
      const double* gvel = (axis == 0) ? gu : (axis == 1) ? gv : gw;
      const double uM = gvel[gM], uP = gvel[gP];
      const double a2 = abs_ct(uP + uM);
      const double tw = (sgi > 0) ? 2.0 : -2.0;
      tP = fma(tw, uP, -a2);
      tM = fma(tw, uM, -a2);
      if (fcout != nullptr) fcout[eb * NFT + ti] = make_double2(tP, tM);
    }
    const dfl gf = df_scale2(df_split(fma(qP, tP, -(qM * tM))), 0.5f);
    sg[ti] = make_float2(gf.hi, gf.lo);
  }
  // phase 1b: x pair values per (line, c < ceil(N/2)): the differences
  // G = q u - F0 by one FMA each, split, then S and Δ in double-float
  for (int t = threadIdx.x; t < nloc * HR * NQ2; t += T) {
    const int le = t / (HR * NQ2);
    const int w = t - le * HR * NQ2;
    const int c = w % HR, r = w / HR;  // c fastest: a warp reads whole lines
    const double* gvel = gu;
    const long long ge = g0 + (long long)le * NP;
    const double f0 = sF0[le * NQ2 + r];
    float2* row = sPl + le * PLANE + r * PADL;
    const int d = 0;
    const int n = line_node(d, r, c);
    const double G1 = fma(qin[ge + n], gvel[ge + n], -f0);
    if (c < H) {
      const int n2 = line_node(d, r, NQ - 1 - c);
      const dfl g1 = df_split(G1);
      const dfl g2 = df_split(fma(qin[ge + n2], gvel[ge + n2], -f0));
      const dfl S = df_add(g1, g2), D = df_sub(g1, g2);
      row[c] = make_float2(S.hi, S.lo);
      row[NQ - 1 - c] = make_float2(D.hi, D.lo);
    } else {
      const dfl M = df_split(G1);
      row[c] = make_float2(M.hi, M.lo);
    }
  }
  __syncthreads();

  // line phases: one thread per line; the x plane then holds the running
  // compensated sums of the nodes, at the node's x-line slot
  const int r = threadIdx.x - (threadIdx.x / NQ2) * NQ2;
  const int le = threadIdx.x / NQ2;
  const bool has_line = le < nloc;
  float2* xpl = sPl + le * PLANE;
  const float2* gl = sg + le * NFT;
  const long long ge = g0 + (long long)le * NP;

  // x lines: r = j + k N; faces -x (3), +x (1) at face node r
  if (has_line) {
    const dfl b0 = df_split(sF0[le * NQ2 + r]);
    float2* row = xpl + r * PADL;
    emu_eo_line<P>(row, sT, b0, f2_df(gl[3 * NFP + r]), f2_df(gl[1 * NFP + r]),
                   [&](int m, const dacc& v) { row[m] = make_float2(v.s, v.c); });
  }
  __syncthreads();

  // y lines: r = i + k N; faces -y (0), +y (2); node (i, m, k) sits in x-line
  // m + k N at slot i
  if (has_line) {
    const int i = r % NQ, k = r / NQ;
    float2 row[NQ];
    double f0;
    emu_eo_pairs<P>(qin, gv, ge + i + NQ2 * k, NQ, row, f0);
    const dfl b0 = df_split(f0);
    emu_eo_line<P>(row, sT + TE, b0, f2_df(gl[r]), f2_df(gl[2 * NFP + r]),
                   [&](int m, const dacc& v) {
                     float2* s = xpl + (m + k * NQ) * PADL + i;
                     dacc acc;
                     acc.s = s->x;
                     acc.c = s->y;
                     dacc_accum(acc, v);
                     *s = make_float2(acc.s, acc.c);
                   });
  }
  __syncthreads();

  // z lines: r = i + j N; faces -z (4), +z (5); finish and RK update
  if (has_line) {
    const int i = r % NQ, j = r / NQ;
    float2 row[NQ];
    double f0;
    emu_eo_pairs<P>(qin, gw, ge + i + NQ * j, NQ2, row, f0);
    const dfl b0 = df_split(f0);
    const dfl c_dt = df_make(a.cdt_hi, a.cdt_lo);
    double* __restrict__ qout = a.q_out;
    const double* __restrict__ q0 = a.q0;
    const double ra = a.a, rb = a.b;
    with_rk_kind(rk_kind(a), [&](auto rkc) {
      constexpr int RK = decltype(rkc)::value;
      emu_eo_line<P>(row, sT + 2 * TE, b0, f2_df(gl[4 * NFP + r]),
                     f2_df(gl[5 * NFP + r]), [&](int m, const dacc& v) {
                       const float2 s = xpl[(j + m * NQ) * PADL + i];
                       dacc acc;
                       acc.s = s.x;
                       acc.c = s.y;
                       dacc_accum(acc, v);
                       const dfl dq = dacc_result(acc);
                       const long long g = ge + i + j * NQ + m * NQ2;
                       if constexpr (RK == kRkTend) {
                         qout[g] = f32_to_f64_bits(dq.hi) + f32_to_f64_bits(dq.lo);
                       } else {
                         const dfl inc = df_mul(c_dt, dq);  // (b*dt)*dqdt
                         const double ih = f32_to_f64_bits(inc.hi), il = f32_to_f64_bits(inc.lo);
                         const double qv = qin[g];
                         if constexpr (RK == kRkFirst)
                           qout[g] = (qv + ih) + il;
                         else
                           qout[g] = fma(ra, q0[g], fma(rb, qv, ih) + il);
                       }
                     });
    });
  }
}

template <int P>
int launch_stage_emu_eo_impl(const StageArgs& a, cudaStream_t st) {
  using C = EmuEoCfg<P>;
  constexpr size_t smem = emu_eo_smem_bytes<P>();
  SDG_TRY(set_kernel_smem((const void*)stage_emu_eo_kernel<P>, (int)smem, false));
  const long long nblk = (a.elem_count + C::EPB - 1) / C::EPB;
  if (nblk <= 0) return SDG_OK;
  if (nblk > 0x7fffffffLL) return fail(SDG_ERR_INVALID_ARG, "too many elements");
  stage_emu_eo_kernel<P><<<(unsigned)nblk, C::THREADS, smem, st>>>(a);
  SDG_CUDA_TRY(cudaGetLastError());
  return SDG_OK;
}

}  // namespace sdg
