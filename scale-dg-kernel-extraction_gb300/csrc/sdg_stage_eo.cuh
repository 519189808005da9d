// Fused RK-stage kernel with the even-odd factorisation of the 1D operators
// (opt type SDG_OPT_EVENODD), for the FP64 form and the FP32-compute form.
//
// On GB300 the FP64 pipe runs at 1/64 of the FP32 rate, so the plain FP64
// stage is bound by its count of FP64 instructions, not by HBM.  This body
// computes the same tendency and stage update as stage_block<P, double> with
// about 30 % fewer FP64 instructions per node; in FP32 it also replaces the
// node body's per-node shared-memory reads of a whole line by one read per
// line value:
//
//  * Centro-antisymmetry of the GLL differentiation matrix,
//    D(N-1-i, N-1-l) = -D(i, l), splits a line's N-term sums into pairs:
//    with S(l) = F(l) + F(N-1-l) and Δ(l) = F(l) - F(N-1-l), l < N/2,
//        e_i = Σ_l E(i,l) S(l) [+ D(i,mid) F(mid)],  o_i = Σ_l O(i,l) Δ(l),
//        out(i) = e_i + o_i,   out(N-1-i) = o_i - e_i,
//    where E / O are the half-sums / half-differences of D's columns l and
//    N-1-l.  A line of N outputs costs N²/2 + 2N operations instead of N².
//  * The lift of a face is a 1D column along the face normal, constant over
//    the tangential nodes, and the + face's column is the mirror of the -
//    face's (Lift_mat of operator_data/p*.dat has both properties to
//    rounding).  With gs = g- + g+ and gd = g- - g+ the two faces of a line
//    join the same pairs: e_i += B(i) gd, o_i += A(i) gs.
//  * Escale, the stage's b*dt and the minus sign of dqdt are folded into the
//    tables when a block stages them, and 0.5*Fscale into the lift columns,
//    so a node's increment is the plain sum of its three line results and
//    the RK update is q_out = b*q + inc (+ a*q0).
//  * The face flux 0.5 Fs (qP VelP - qM VelM - α (qP - qM)) is formed as
//    qP (2VelP - 2α) - qM (2VelM - 2α) with 2α = |uP + uM| (the normal sign
//    applied through the constant ±2): five FP64 operations per face node.
//    Three of them form the velocity factors tP = ±2VelP - 2α and tM, which
//    every stage of one solver call shares (the velocity cannot change
//    within a call): the call's first stage stores them (fc_out) and every
//    later stage reads them (fc_in), two operations a face node there.
//
// Thread layout: phase 0 and the face flux run one thread per node / face
// node as in stage_block; the three contraction phases run one thread per
// line (N² lines per element and direction).  The x phase writes its line
// results over F_x, the y phase adds into them and the z phase finishes the
// node: every phase touches only its own line's nodes, and a barrier
// separates the phases.
//
// The summation order is neither GENERAL's nor OPT1's; the result agrees
// with both to rounding (the parity tests hold it to the same tolerance).
// The host builds the E / O / lift tables only after checking the operator
// symmetries; operators without them are refused for this opt type.
#pragma once

#include "sdg_stage.cuh"

namespace sdg {

template <int P>
struct EoShape {
  static constexpr int N = P + 1;
  static constexpr int H = N / 2;          // pairs (l, N-1-l)
  static constexpr int HR = (N + 1) / 2;   // output rows incl. the middle row
  static constexpr int ODD = N & 1;
  static constexpr int OFF_E = 0;                      // E(i,l), i < H, l < H
  static constexpr int OFF_O = H * H;                  // O(i,l), i < HR, l < H
  static constexpr int OFF_DM = OFF_O + HR * H;        // D(i,mid), i < H (odd N)
  static constexpr int OFF_A = OFF_DM + ODD * H;       // lift sym part, i < HR
  static constexpr int OFF_B = OFF_A + HR;             // lift antisym part, i < H
  static constexpr int TE = OFF_B + H;                 // entries per direction
};

// Threads per line in the line phases: the FP32 body splits a line's output
// pairs between two threads (each forms the line's pair sums itself), which
// halves the registers a thread needs and doubles the warps that hide memory
// latency; at low orders a line has one or two output pairs, and one thread
// a line measured faster on GB300 up to p = 3 in the single-box kernel (p = 3:
// 91.8 against 72.5 GDOF-updates/s).  The FP64 body is bound by the FP64 pipe
// and keeps one.  The batched kernels pick their own count (batch_eo_parts).
// At p = 4 and 6 one thread a line measured faster (77.5 against 70.0
// GDOF-updates/s at p = 4 with 256 threads and six blocks an SM; 77.3 against
// 69.1 at p = 6 with four); likewise at p = 5 with five blocks of 256 threads
// (81.5 against 79.6 for four elements on 256 threads with two threads a
// line) and at p = 11..14 with the block counts of eo_min_blocks (92.3
// against 90.0, 88.4 against 80.1, 87.9 against 78.2, 82.7 against 72.1);
// level or slower at p = 8..10 and 15.
template <int P, typename CT>
__host__ __device__ constexpr int eo_parts() {
  return (sizeof(CT) == 4 && P >= 7 && (P < 11 || P > 14)) ? 2 : 1;
}

// Lines of a block: 256, or 128 for the FP32 body at p = 7, 9 and 10, where
// twice as many half-size blocks (the same 64 warps an SM) measured 1.04-1.05x
// on GB300 (108 against 103 GDOF-updates/s at p = 7; 0.95x at p = 8), and for
// the FP64 body at p = 7 (eight blocks of 128 threads for four of 256, the
// same 61 registers: 19.81 against 19.68 GDOF-updates/s; at p = 1..5 the
// same change measured 0.97-1.008x).
template <int P, typename CT>
__host__ __device__ constexpr int eo_lines() {
  return ((sizeof(CT) == 4 && (P == 7 || P == 9 || P == 10)) || (sizeof(CT) == 8 && P == 7))
             ? 128
             : 256;
}

template <int P, typename CT>
__host__ __device__ constexpr bool eo_exact() {
  return sizeof(CT) == 4 && (P == 11 || P == 12);
}

template <int P, typename CT = double>
struct EoCfg {
  // FP32 at p = 11 and 12: one element a block, the block sized to its
  // lines instead of 256 lines of which 144 / 169 had work; measured on
  // GB300 with two threads a line 90.2 against 86.7 and 80.3 against 74.6
  // GDOF-updates/s (now one thread a line, eo_parts: 160 and 192 threads).
  // At p = 13 and 14 the 256-line shape stays faster (78.2 against 77.3,
  // 72.1 against 71.6 with two threads a line), at p = 9 level (87.0 against
  // 86.5), and the FP64 form at p = 11..13, bound by its FP64 pipe, level.
  static constexpr bool EXACT = eo_exact<P, CT>();
  static constexpr int LINES = eo_lines<P, CT>();
  static constexpr int THREADS = EXACT ? ((Ord<P>::NQ2 * eo_parts<P, CT>() + 31) / 32) * 32
                                       : LINES * eo_parts<P, CT>();
  static constexpr int EPB = EXACT ? 1 : (LINES / Ord<P>::NQ2) > 0 ? LINES / Ord<P>::NQ2 : 1;
};

// Dynamic shared memory of one block with nloc elements: the three scaled
// direction tables, then per element the arrays below and the 6 Nfp face
// fluxes, then the neighbour indices.
// The FP64 body does not stage q: the face flux and the RK update read it
// from global memory (L1 / L2 hits after phase 0), which saves shared memory
// for a fourth resident block.
template <typename CT>
__host__ __device__ constexpr bool eo_stages_q() {
  return sizeof(CT) == 4;
}

// The FP64 body keeps one array: the x lines' pair values, then the sums; the
// y and z line threads form their lines' pair values from q and v / w in
// cache.  That leaves room for four resident blocks.  The FP32 body keeps q
// (FP32), F_x and the line-result sums (in their own array, since two threads
// share a line and one may write before the other has read), and either
// stages F_y and F_z as well or (FLY) has the y and z line threads form
// F = q v / q w from the staged q and the velocity in cache: two arrays less,
// which keeps more blocks resident at high orders, for two extra velocity
// reads per line node.
template <int P, typename CT, bool FLY = false, int PARTS_SET = 0>
__host__ __device__ constexpr size_t eo_block_smem(int nloc) {
  using O = Ord<P>;
  constexpr int parts = PARTS_SET > 0 ? PARTS_SET : eo_parts<P, CT>();
  constexpr int arrays =
      sizeof(CT) == 8 ? 1 : (eo_stages_q<CT>() ? 2 : 1) + (FLY ? 0 : 2) + (parts > 1 ? 1 : 0);
  return sizeof(CT) * (size_t)(3 * EoShape<P>::TE + nloc * (arrays * O::NP + O::NFT)) +
         sizeof(int) * 6 * (size_t)nloc;
}

// Starts moving the 128-byte line holding p into L2 (no register, no wait).
__device__ __forceinline__ void prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

__device__ __forceinline__ double abs_ct(double x) {
  return __longlong_as_double(__double_as_longlong(x) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ float abs_ct(float x) { return fabsf(x); }

// One line: F (stride S) holds the line's N volume fluxes, T the direction's
// scaled tables, gm / gp the face fluxes of the line's - and + faces.  The
// N results go to emit(m, value) after all reads of F.
// With PARTS threads on a line, thread `part` produces the pairs of rows
// [part * RPP, (part + 1) * RPP) (RPP = ceil(H / PARTS)) and the last part the
// middle row of an odd N.
// PAIRED: F holds S(l) at l and Δ(l) at N-1-l (l < N/2) and, for odd N, F
// at the middle, formed when the line was loaded; otherwise F holds the N
// fluxes and the pair values are formed here.
// Load(l) returns the line's value at node l (l < N).
template <int P, int PARTS, bool PAIRED, typename CT, typename Load, typename Emit>
__device__ __forceinline__ void eo_line_f(Load&& F, const CT* __restrict__ T, CT gm, CT gp,
                                          int part, Emit&& emit) {
  using Sh = EoShape<P>;
  constexpr int N = Sh::N, H = Sh::H;
  constexpr int RPP = (H + PARTS - 1) / PARTS;
  CT s[H], d[H];
#pragma unroll
  for (int l = 0; l < H; l++) {
    const CT lo = F(l), hi = F(N - 1 - l);
    if constexpr (PAIRED) {
      s[l] = lo;
      d[l] = hi;
    } else {
      s[l] = lo + hi;
      d[l] = lo - hi;
    }
  }
  CT fm = CT(0);
  if constexpr (Sh::ODD != 0) fm = F(H);
  const CT gs = gm + gp, gd = gm - gp;
  // rows unrolled up to p = 7 in FP32 and p = 4 in FP64; above that a rolled
  // loop keeps the 2H line values and the row sums within the register budget
  // (64 registers for four resident FP64 blocks of 256 threads)
  constexpr int kRowUnroll = (N <= (sizeof(CT) == 8 ? 5 : 8)) ? RPP : 1;
#pragma unroll kRowUnroll
  for (int ii = 0; ii < RPP; ii++) {
    const int i = part * RPP + ii;
    if (PARTS > 1 && i >= H) break;
    CT e = T[Sh::OFF_E + i * H] * s[0];
#pragma unroll
    for (int l = 1; l < H; l++) e = fma(T[Sh::OFF_E + i * H + l], s[l], e);
    if constexpr (Sh::ODD != 0) e = fma(T[Sh::OFF_DM + i], fm, e);
    e = fma(T[Sh::OFF_B + i], gd, e);
    CT o = T[Sh::OFF_O + i * H] * d[0];
#pragma unroll
    for (int l = 1; l < H; l++) o = fma(T[Sh::OFF_O + i * H + l], d[l], o);
    o = fma(T[Sh::OFF_A + i], gs, o);
    emit(i, e + o);
    emit(N - 1 - i, o - e);
  }
  if (Sh::ODD != 0 && part == PARTS - 1) {
    CT o = T[Sh::OFF_O + H * H] * d[0];
#pragma unroll
    for (int l = 1; l < H; l++) o = fma(T[Sh::OFF_O + H * H + l], d[l], o);
    o = fma(T[Sh::OFF_A + H], gs, o);
    emit(H, o);
  }
}

template <int P, int S, int PARTS, bool PAIRED, typename CT, typename Emit>
__device__ __forceinline__ void eo_line(const CT* F, const CT* __restrict__ T, CT gm, CT gp,
                                        int part, Emit&& emit) {
  eo_line_f<P, PARTS, PAIRED, CT>([&](int l) { return F[l * S]; }, T, gm, gp, part, emit);
}

// Pair values of one line from q and the axis velocity in global memory (FP64
// body): S(c) = F(c) + F(N-1-c) and Δ(c) = F(c) - F(N-1-c) with F = q u, as
// P' = q' u' and fma(q, u, ±P') -- three operations a pair instead of four.
template <int P>
__device__ __forceinline__ void eo_pairs_f64(const double* __restrict__ q,
                                             const double* __restrict__ vel, long long g,
                                             int stride, double* row) {
  using Sh = EoShape<P>;
  constexpr int N = Sh::N, H = Sh::H;
#pragma unroll
  for (int c = 0; c < H; c++) {
    const long long a = g + (long long)c * stride, b = g + (long long)(N - 1 - c) * stride;
    const double q1 = q[a], u1 = vel[a];
    const double p2 = q[b] * vel[b];
    row[c] = fma(q1, u1, p2);
    row[N - 1 - c] = fma(q1, u1, -p2);
  }
  if constexpr (Sh::ODD != 0) row[H] = q[g + (long long)H * stride] * vel[g + (long long)H * stride];
}

// One block advances elements [eb, eb + nloc) through one stage with the
// even-odd body.  CT = double: FP64 throughout (tables scaled by eo_sD /
// eo_sL).  CT = float: the FP32-compute form (FP32 tables, velocity and
// sums, scaled by eo_sDf / eo_sLf), with the increment widened by bits and
// the RK combination in FP64.  Block size and nloc are runtime values, so the
// batched persistent kernel can use the same body.
// PREF (FP32 body): start q0 towards L2 in phase 0 and unroll the staging
// loop by 4, so more loads are in flight per warp.  (Four nodes a thread as
// 16-byte loads measured 0.93-0.98x at p = 5..11: the stores of four
// consecutive nodes a thread hit the same shared-memory banks.)  Measured on GB300 for the
// single-box kernel: 1.03-1.06x at p >= 4 (103 GDOF-updates/s at p = 7),
// 0.95x at p = 1; in the batched kernel it was 0.8-0.9x, so it stays off there.
template <int P, typename CT, int RKFIX = -1, bool FLY = false, bool PREF = false,
          int PARTS_SET = 0>
__device__ __forceinline__ void stage_eo_block(const StageArgs& a, long long eb, int nloc,
                                               unsigned char* smem) {
  using O = Ord<P>;
  using Sh = EoShape<P>;
  constexpr int NQ = O::NQ, NQ2 = O::NQ2, NP = O::NP, NFP = O::NFP, NFT = O::NFT;
  constexpr int TE = Sh::TE;
  constexpr bool kF64 = sizeof(CT) == 8;
  const int T = blockDim.x;
  CT* sT = reinterpret_cast<CT*>(smem);  // 3 directions x TE
  constexpr bool kSQ = eo_stages_q<CT>();
  CT* sq = sT + 3 * TE;      // q (FP32 body only)
  CT* sFx = sq + (kSQ ? nloc * NP : 0);  // F_x (FP64: x pair values), then the sums
  constexpr bool kSYZ = !kF64 && !FLY;    // F_y, F_z staged (FP32 only)
  CT* sFy = sFx + (kSYZ ? nloc * NP : 0);
  CT* sFz = sFy + (kSYZ ? nloc * NP : 0);
  constexpr int PARTS = PARTS_SET > 0 ? PARTS_SET : eo_parts<P, CT>();
  CT* sAcc = (PARTS > 1) ? sFz + nloc * NP : sFx;  // line-result sums
  CT* sf = ((PARTS > 1) ? sAcc : sFz) + nloc * NP;   // after the last array
  int* snb = reinterpret_cast<int*>(sf + nloc * NFT);

  const double* __restrict__ qin = a.q_in;
  const CT* __restrict__ gu = static_cast<const CT*>(a.u);
  const CT* __restrict__ gv = static_cast<const CT*>(a.v);
  const CT* __restrict__ gw = static_cast<const CT*>(a.w);
  const CT* __restrict__ tab = static_cast<const CT*>(a.D);
  const long long g0 = eb * NP;

  // phase 0: scaled tables, neighbours, q and F_d = q * u_d.  The factors
  // are picked by selects, not by a runtime array index, so that the
  // argument struct can stay in registers in the batched kernel.
  CT fD[3], fL[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if constexpr (kF64) {
      fD[d] = a.eo_sD[d];
      fL[d] = a.eo_sL[d];
    } else {
      fD[d] = a.eo_sDf[d];
      fL[d] = a.eo_sLf[d];
    }
  }
  for (int t = threadIdx.x; t < 3 * TE; t += T) {
    const int dir = t / TE, w = t - dir * TE;
    const CT sd = (dir == 0) ? fD[0] : (dir == 1) ? fD[1] : fD[2];
    const CT sl = (dir == 0) ? fL[0] : (dir == 1) ? fL[1] : fL[2];
    sT[t] = tab[t] * ((w < Sh::OFF_A) ? sd : sl);
  }
  for (int t = threadIdx.x; t < 6 * nloc; t += T)
    snb[t] = (int)neighbor(a.box, eb + t / 6, t % 6);
  if constexpr (kF64) {
    // x pair values: one task per (element, x line, c < ceil(N/2)), c fastest
    constexpr int HR = Sh::HR, H = Sh::H;
    for (int t = threadIdx.x; t < nloc * NQ2 * HR; t += T) {
      const int le = t / (NQ2 * HR), w = t - le * NQ2 * HR;
      const int r = w / HR, c = w - r * HR;
      const long long g = g0 + (long long)le * NP + (long long)r * NQ;
      CT* row = sFx + le * NP + r * NQ;
      if (c < H) {
        const double q1 = qin[g + c], u1 = gu[g + c];
        const double p2 = qin[g + NQ - 1 - c] * gu[g + NQ - 1 - c];
        row[c] = fma(q1, u1, p2);
        row[NQ - 1 - c] = fma(q1, u1, -p2);
      } else {
        row[c] = qin[g + c] * gu[g + c];
      }
    }
  } else {
    auto stage_node = [&](int t) {
      const CT qq = to_ct<CT>(qin[g0 + t]);
      if constexpr (kSQ) sq[t] = qq;
      sFx[t] = qq * gu[g0 + t];
      if constexpr (kSYZ) {
        sFy[t] = qq * gv[g0 + t];
        sFz[t] = qq * gw[g0 + t];
      }
    };
    if constexpr (PREF) {
      // q0, read only by the last phase's RK update, starts towards L2 now
      if (rk_kind(a) == kRkGeneral)
        for (int t = 16 * threadIdx.x; t < nloc * NP; t += 16 * T) prefetch_l2(a.q0 + g0 + t);
#pragma unroll 4
      for (int t = threadIdx.x; t < nloc * NP; t += T) stage_node(t);
    } else {
      for (int t = threadIdx.x; t < nloc * NP; t += T) stage_node(t);
    }
  }
  __syncthreads();

  // phase 1: face fluxes qP (2VelP - 2α) - qM (2VelM - 2α), unscaled.  The
  // velocity factors tP = ±2VelP - 2α and tM come from fc_in when a stage
  // before this one in the step stored them (FP64 body).
  const double2* __restrict__ fcin = reinterpret_cast<const double2*>(a.fc_in);
  double2* __restrict__ fcout = reinterpret_cast<double2*>(a.fc_out);
  // tasks face-major below p = 5 (FaceTasks)
  const FaceTasks<NQ> ftask(nloc);
  for (int t = threadIdx.x; t < nloc * NFT; t += T) {
    int le, f, fp;
    ftask.map(t, le, f, fp);
    const int r = f * NFP + fp;
    const int ti = le * NFT + r;  // the task's element-major index
    int nM, nP, axis, sg;
    face_nodes<NQ>(f, fp % NQ, fp / NQ, nM, nP, axis, sg);
    const long long gM = g0 + (long long)le * NP + nM;
    const long long gP = (long long)snb[6 * le + f] * NP + nP;
    CT qM;
    if constexpr (kSQ)
      qM = sq[le * NP + nM];
    else
      qM = to_ct<CT>(qin[gM]);
    const CT qP = to_ct<CT>(qin[gP]);
    CT tP, tM;
    if (kF64 && fcin != nullptr) {
      const double2 c = fcin[eb * NFT + ti];
      tP = CT(c.x);
      tM = CT(c.y);
    } else {
      const CT* gvel = (axis == 0) ? gu : (axis == 1) ? gv : gw;
      const CT uM = gvel[gM], uP = gvel[gP];
      const CT a2 = abs_ct(uP + uM);
      const CT tw = (sg > 0) ? CT(2) : CT(-2);
      tP = fma(tw, uP, -a2);
      tM = fma(tw, uM, -a2);
      if (kF64 && fcout != nullptr) fcout[eb * NFT + ti] = make_double2(tP, tM);
    }
    sf[ti] = fma(qP, tP, -(qM * tM));
  }
  __syncthreads();

  // phase 2x: lines along i, faces -x (3) and +x (1); results into the sums
  // (over F_x itself when one thread owns the line)
  for (int t = threadIdx.x; t < nloc * NQ2 * PARTS; t += T) {
    const int part = t % PARTS, lt = t / PARTS;
    const int le = lt / NQ2, r = lt - le * NQ2;
    const CT* F = sFx + le * NP + r * NQ;
    CT* acc = sAcc + le * NP + r * NQ;
    const CT* fl = sf + le * NFT + r;
    eo_line<P, 1, PARTS, kF64>(F, sT, fl[3 * NFP], fl[1 * NFP], part,
                         [&](int m, CT v) { acc[m] = v; });
  }
  __syncthreads();

  // phase 2y: lines along j, faces -y (0) and +y (2); added into the sums
  for (int t = threadIdx.x; t < nloc * NQ2 * PARTS; t += T) {
    const int part = t % PARTS, lt = t / PARTS;
    const int le = lt / NQ2, r = lt - le * NQ2;
    const int off = le * NP + (r % NQ) + (r / NQ) * NQ2;
    CT* acc = sAcc + off;
    const CT* fl = sf + le * NFT + r;
    if constexpr (kF64) {
      double row[NQ];
      eo_pairs_f64<P>(qin, gv, g0 + off, NQ, row);
      eo_line<P, 1, PARTS, true>(row, sT + TE, fl[0], fl[2 * NFP], part,
                                 [&](int m, CT v) { acc[m * NQ] += v; });
    } else if constexpr (kSYZ) {
      eo_line<P, NQ, PARTS, false>(sFy + off, sT + TE, fl[0], fl[2 * NFP], part,
                                   [&](int m, CT v) { acc[m * NQ] += v; });
    } else {
      // __fmul_rn: the product is rounded before the pair sums, exactly as a
      // staged F_y would be (no contraction into an FMA), so both forms and
      // the batched kernels give the same bits
      const CT* qr = sq + off;
      const CT* vr = gv + g0 + off;
      eo_line_f<P, PARTS, false, CT>([&](int l) { return __fmul_rn(qr[l * NQ], vr[l * NQ]); },
                                     sT + TE,
                                     fl[0], fl[2 * NFP], part,
                                     [&](int m, CT v) { acc[m * NQ] += v; });
    }
  }
  __syncthreads();

  // phase 2z: lines along k, faces -z (4) and +z (5); finish the node and the
  // RK update q_out = b*q + inc (+ a*q0).  The lambda captures plain locals,
  // not the argument struct, which would otherwise live in local memory when
  // the batched kernel builds it per work item.
  double* __restrict__ qout = a.q_out;
  const double* __restrict__ q0 = a.q0;
  const double rk_a = a.a, rk_b = a.b;
  with_rk_kind<RKFIX>(rk_kind(a), [&](auto rkc) {
    constexpr int RK = decltype(rkc)::value;
    for (int t = threadIdx.x; t < nloc * NQ2 * PARTS; t += T) {
      const int part = t % PARTS, lt = t / PARTS;
      const int le = lt / NQ2, r = lt - le * NQ2;
      const int off = le * NP + r;
      const CT* fl = sf + le * NFT + r;
      auto emitz = [&](int m, CT v) {
        const int n = off + m * NQ2;
        const long long g = g0 + n;
        double inc;
        if constexpr (kF64)
          inc = sAcc[n] + v;
        else
          inc = f32_to_f64_bits(sAcc[n] + v);
        if constexpr (RK == kRkTend)
          qout[g] = inc;
        else
          qout[g] = rk_combine<RK>(inc, qin[g], RK == kRkGeneral ? q0[g] : 0.0, rk_a, rk_b);
      };
      if constexpr (kF64) {
        double row[NQ];
        eo_pairs_f64<P>(qin, gw, g0 + off, NQ2, row);
        eo_line<P, 1, PARTS, true>(row, sT + 2 * TE, fl[4 * NFP], fl[5 * NFP], part, emitz);
      } else if constexpr (kSYZ) {
        eo_line<P, NQ2, PARTS, false>(sFz + off, sT + 2 * TE, fl[4 * NFP], fl[5 * NFP], part,
                                      emitz);
      } else {
        const CT* qr = sq + off;
        const CT* wr = gw + g0 + off;
        eo_line_f<P, PARTS, false, CT>([&](int l) { return __fmul_rn(qr[l * NQ2], wr[l * NQ2]); },
                                       sT + 2 * TE, fl[4 * NFP], fl[5 * NFP], part, emitz);
      }
    }
  });
}

// Resident blocks an SM.  FP32, two threads a line (512 threads, or 256 at
// p = 7, 9, 10 with twice the blocks): the body issues few instructions per
// byte and needs warps to hide memory latency, so the registers are capped at
// 32 for 64 warps (measured 1.0-1.16x the three-block build, 100 against 91.5
// GDOF-updates/s at p = 7); at p = 15 shared memory admits three blocks and
// the cap would only spill.  One thread a line (p <= 6 and 11..14): the
// counts below, each measured on GB300 against its neighbours.
// FP64: four or five blocks of 256 threads (registers capped at 64 or 48): a
// block in its load or flux phase leaves the others feeding the FP64 pipe.
// Five measured faster on GB300 at most orders once stages 2-3 read the face
// factors (1.02-1.06x up to p = 4, 1.005-1.013x at p = 6 and 8..13, 48
// registers with small spills) and four at p = 5, 7, 14 and 15 (by 0.2-1.1 %).
// At p = 1 eight blocks (32 registers, 68 bytes of spills) measured 20.5
// against 19.8 GDOF-updates/s for five (20.4 for six); at p = 2 six were level.
// At p = 7 the blocks have 128 threads (eo_lines), so four blocks' worth of
// warps is eight blocks (ten, at 48 registers with spills: 19.75).
template <int P, typename CT>
__host__ __device__ constexpr int eo_min_blocks() {
  if (sizeof(CT) == 8) return P == 7 ? 8 : (P == 5 || P >= 14) ? 4 : P == 1 ? 8 : 5;
  if (P == 4) return 6;  // 40 registers, one thread a line (above)
  if (P == 5) return 5;  // 48 registers, one thread a line
  // one thread a line from p = 11 to 14 (eo_parts); p = 11, 12 in blocks
  // sized to one element's lines (EoCfg: 160 and 192 threads)
  if (P == 11) return 5;
  if (P == 12 || P == 13) return 6;
  if (P == 14) return 4;
  return (P <= 3 || eo_lines<P, CT>() == 128) ? 8 : P <= 12 ? 4 : 3;
}

// FP32 single-box kernel: F_y / F_z formed on the fly (FLY) at the orders
// where that measured faster on GB300 (1.07-1.18x at p = 10, 13 and 15, even
// at 12 and 14); staging them is faster below (up to 1.15x at p = 6;
// rechecked with the current shapes at p = 4, 6 and 8: FLY 0.92-0.99x).
template <int P>
__host__ __device__ constexpr bool eo_fly_single() {
  return P == 10 || P >= 12;
}

template <int P, typename CT>
__global__ void __launch_bounds__(EoCfg<P, CT>::THREADS, eo_min_blocks<P, CT>())
    stage_eo_kernel(const StageArgs a) {
  constexpr int EPB = EoCfg<P, CT>::EPB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const long long eb = a.elem_begin + (long long)blockIdx.x * EPB;
  const long long eend = a.elem_begin + a.elem_count;
  const int nloc = (int)((eend - eb) < EPB ? (eend - eb) : EPB);
  if (nloc <= 0) return;
  stage_eo_block<P, CT, -1, eo_fly_single<P>(), (P >= 4)>(a, eb, nloc, smem_raw);
}

template <int P, typename CT>
int launch_stage_eo_impl(const StageArgs& a, cudaStream_t st) {
  constexpr size_t smem = eo_block_smem<P, CT, eo_fly_single<P>()>(EoCfg<P, CT>::EPB);
  SDG_TRY(set_kernel_smem((const void*)stage_eo_kernel<P, CT>, (int)smem, true));
  const long long nblk = (a.elem_count + EoCfg<P, CT>::EPB - 1) / EoCfg<P, CT>::EPB;
  if (nblk <= 0) return SDG_OK;
  if (nblk > 0x7fffffffLL) return fail(SDG_ERR_INVALID_ARG, "too many elements");
  stage_eo_kernel<P, CT><<<(unsigned)nblk, EoCfg<P, CT>::THREADS, smem, st>>>(a);
  SDG_CUDA_TRY(cudaGetLastError());
  return SDG_OK;
}

}  // namespace sdg
