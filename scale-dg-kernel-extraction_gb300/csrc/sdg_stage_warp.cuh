// Warp-cooperative forms of the FP32-compute even-odd stage for p = 2 and 3.
//
// At these orders an element has 27 or 64 nodes and lines of 3 or 4 nodes.
// The block-cooperative body (stage_eo_block) distributes that little work
// through shared memory, per-task index arithmetic and four barriers and is
// issue-bound (63 % issue at p = 2 with DRAM at 25 % of its peak).  Here the
// lanes of a warp share a few elements and exchange line values and face
// fluxes by warp shuffle: no shared memory, no barrier.
//
//  * p = 2, column form: nine lanes an element, three elements a warp; a
//    lane holds an x line (three contiguous nodes) and both of its x faces,
//    the y and z lines come by shuffle.  Measured on GB300 at 85^3: 110.8
//    GDOF-updates/s against 71.4 for the block body.
//  * p = 3, node form: a warp an element, lane L holding nodes L and L + 32.
//    105.2 against 96.4 at 64^3; the column form (sixteen lanes an element,
//    four nodes a lane) needs 128 registers a thread and measured 96.5.
//
// A face node's lane forms the face flux itself from its own values and the
// neighbour's opposite node (a global gather, an L1 / L2 hit).  Every lane
// keeps the table entries of its own rows in registers (read once per
// thread), and a warp strides over many elements, so that set-up is paid
// once.
//
// The arithmetic is stage_eo_block<P, float>'s operation for operation --
// F = q u rounded (__fmul_rn), the five-operation face flux, eo_line_f's pair
// sums, its e / o chains in the same order with the same scaled FP32 table
// entries, e + o / o - e / o (the middle row of odd N, written o + (-0), an
// identity also for o = ±0), the line results added in x, y, z order, the
// widened increment and the FP64 RK update -- so the result equals that
// body's bit for bit, and the batched kernels, which keep the block body,
// stay bit-identical to the single-box solver (tested).
#pragma once

#include "sdg_stage_eo.cuh"

namespace sdg {

constexpr unsigned kFullMask = 0xffffffffu;

// An element and its coordinates in the box (e = ex + NeX (ey + NeY ez)).
struct ElemPos {
  int e, ex, ey, ez;
};

// Element coordinates by multiply-high with ceil(2^32 / NeX) and
// ceil(2^32 / NeY), exact for e NeX < 2^32 and e NeY < 2^32 (the quotient's
// error e r / (d 2^32), r < d, stays below 1 / d) and d > 1 (the constant of
// d = 1 does not fit 32 bits); other boxes divide.  The
// element index is warp-uniform, so either form is a few uniform
// instructions an element instead of two 32-bit divisions.
struct ElemIndexer {
  unsigned nx, ny, mx, my;
  bool fast;
  __device__ __forceinline__ ElemIndexer(const Box& b, long long end)
      : nx((unsigned)b.NeX), ny((unsigned)b.NeY),
        mx(0xFFFFFFFFu / (unsigned)b.NeX + 1u), my(0xFFFFFFFFu / (unsigned)b.NeY + 1u),
        fast(b.NeX > 1 && b.NeY > 1 &&
             end * (long long)(b.NeX > b.NeY ? b.NeX : b.NeY) < (1LL << 32)) {}
  __device__ __forceinline__ ElemPos pos(long long e64) const {
    ElemPos p;
    const unsigned e = (unsigned)e64;  // element counts are below 2^31
    const unsigned rxy = fast ? __umulhi(e, mx) : e / nx;
    const unsigned rz = fast ? __umulhi(rxy, my) : rxy / ny;
    p.e = (int)e;
    p.ex = (int)(e - rxy * nx);
    p.ey = (int)(rxy - rz * ny);
    p.ez = (int)rz;
    return p;
  }
};

// The element across the - (minus) or + face of axis D, with periodic wrap:
// the element neighbor() returns for faces 3 / 1, 0 / 2 and 4 / 5.
template <int D>
__device__ __forceinline__ int elem_across(const Box& b, const ElemPos& p, bool minus) {
  if constexpr (D == 0) {
    const int x = minus ? (p.ex == 0 ? b.NeX - 1 : p.ex - 1) : (p.ex == b.NeX - 1 ? 0 : p.ex + 1);
    return p.e + (x - p.ex);
  } else if constexpr (D == 1) {
    const int y = minus ? (p.ey == 0 ? b.NeY - 1 : p.ey - 1) : (p.ey == b.NeY - 1 ? 0 : p.ey + 1);
    return p.e + (y - p.ey) * b.NeX;
  } else {
    const int z = minus ? (p.ez == 0 ? b.NeZ - 1 : p.ez - 1) : (p.ez == b.NeZ - 1 ? 0 : p.ez + 1);
    return p.e + (z - p.ez) * (b.NeX * b.NeY);
  }
}

// The neighbour's values at the node across a face: q (converted to FP32
// where it is used) and the axis velocity.
struct FaceIn {
  double qP;
  float uP;
};

// Gathers them for node n (line position 0 on the - face, NQ-1 on the + face
// of axis D): the neighbour's node with the same tangential indices.  A lane
// whose node is on neither face (face = false) loads its own node instead, so
// that every lane issues the same loads without a branch; its values are
// never read.
template <int P, int D>
__device__ __forceinline__ FaceIn face_gather(const StageArgs& a, const float* __restrict__ gvel,
                                              const ElemPos& p, int n, bool minus,
                                              bool face = true) {
  using O = Ord<P>;
  constexpr int S = D == 0 ? 1 : D == 1 ? O::NQ : O::NQ2;
  const int nb = face ? elem_across<D>(a.box, p, minus) : p.e;
  const int nP = !face ? n : minus ? n + (O::NQ - 1) * S : n - (O::NQ - 1) * S;
  const long long gP = (long long)nb * O::NP + nP;
  return FaceIn{a.q_in[gP], gvel[gP]};
}

// Face flux qP (±2 uP - |uP + uM|) - qM (±2 uM - |uP + uM|) from the node's
// own qM, uM and the gathered neighbour values.
__device__ __forceinline__ float face_flux(const FaceIn& in, bool minus, float qM, float uM) {
  const float qP = to_ct<float>(in.qP);
  const float uP = in.uP;
  const float a2 = fabsf(uP + uM);
  const float tw = minus ? -2.0f : 2.0f;
  const float tP = fmaf(tw, uP, -a2);
  const float tM = fmaf(tw, uM, -a2);
  return fmaf(qP, tP, -(qM * tM));
}

// One lane's row of a direction's scaled tables: E(row, :), O(row, :),
// D(row, mid) and the lift entries B(row), A(row); `add` says how the row's
// e joins o for this lane's node (+1: e + o, -1: o - e, 0: the middle row,
// o alone).  For the middle row of odd N, O and A come from row H.
template <int P>
struct WarpRow {
  static constexpr int H = EoShape<P>::H;
  float E[H], Od[H], DM, B, A;
  int add;

  __device__ __forceinline__ void load(const float* __restrict__ tab, int dir, float sD, float sL,
                                       int l) {
    using Sh = EoShape<P>;
    constexpr int N = Sh::N;
    const float* t = tab + dir * Sh::TE;
    const bool mid = Sh::ODD != 0 && l == H;
    const int row = l < H ? l : N - 1 - l;
    const int erow = mid ? 0 : row;
    const int orow = mid ? H : row;
#pragma unroll
    for (int c = 0; c < H; c++) {
      E[c] = t[Sh::OFF_E + erow * H + c] * sD;
      Od[c] = t[Sh::OFF_O + orow * H + c] * sD;
    }
    DM = Sh::ODD != 0 ? t[Sh::OFF_DM + erow] * sD : 0.0f;
    B = t[Sh::OFF_B + erow] * sL;
    A = t[Sh::OFF_A + orow] * sL;
    add = mid ? 0 : (l < H ? 1 : -1);
  }

  // The lane's output of a line with values F(0..N-1) and face fluxes gm, gp.
  __device__ __forceinline__ float apply(const float (&F)[EoShape<P>::N], float gm,
                                         float gp) const {
    using Sh = EoShape<P>;
    constexpr int N = Sh::N;
    float s[H], d[H];
#pragma unroll
    for (int c = 0; c < H; c++) {
      s[c] = F[c] + F[N - 1 - c];
      d[c] = F[c] - F[N - 1 - c];
    }
    const float gs = gm + gp, gd = gm - gp;
    float e = E[0] * s[0];
#pragma unroll
    for (int c = 1; c < H; c++) e = fmaf(E[c], s[c], e);
    if constexpr (Sh::ODD != 0) e = fmaf(DM, F[H], e);
    e = fmaf(B, gd, e);
    float o = Od[0] * d[0];
#pragma unroll
    for (int c = 1; c < H; c++) o = fmaf(Od[c], d[c], o);
    o = fmaf(A, gs, o);
    const float ea = add > 0 ? e : add < 0 ? -e : -0.0f;
    return o + ea;
  }
};

template <int P>
struct WarpCfg {
  static constexpr int THREADS = 256;
  static constexpr int WARPS = THREADS / 32;
  // resident blocks an SM the registers are capped for, and whether a warp
  // issues the next elements' loads before computing the current ones.
  // Measured on GB300: p = 2 (column form) 110.8 GDOF-updates/s with two
  // blocks and the prefetch (128 registers), 99.4 / 92.0 / 81.9 with two,
  // three, four blocks without; p = 3 (node form) 105.8 with three blocks
  // (80 registers) against 103.9 with four and 99.7 with two and the prefetch.
  static constexpr int MIN_BLOCKS = P == 2 ? 2 : 3;
  static constexpr bool PREFETCH = P == 2;
};

// Column form (used at p = 2): NQ^2 lanes an element, 32 / NQ^2 elements a
// warp (three at p = 2).  Lane NQ^2 s + c (c = j + NQ k) holds the x
// line (0..NQ-1, j, k) of element e0 + s, nodes NQ c .. NQ c + NQ-1: the
// warp's loads are contiguous rows, the x line and both of its faces are the
// lane's own, a y line (i, 0..NQ-1, k) lies across lanes NQ^2 s + NQ k + j'
// and a z line across lanes NQ^2 s + j + NQ k' (slot i of each).  At p = 2
// lanes 27..31 shadow lane 26 and store nothing.
//
// Every global load of the warp's elements is issued together -- the nodes'
// q, q0 and velocity and the neighbour values of the faces the lane's nodes
// lie on (their addresses depend only on the element index) -- so a set of
// elements costs one memory round trip; with PREFETCH the next set's loads
// are in flight while this one is computed.
template <int P>
struct ColIn {
  static constexpr int NQ = P + 1;
  double q[NQ], q0[NQ];
  float u[NQ], v[NQ], w[NQ];
  FaceIn xm, xp, y[NQ], z[NQ];
};

template <int P>
struct ColShape {
  static constexpr int NQ = P + 1, NQ2 = NQ * NQ, NP = NQ * NQ2;
  static constexpr int EPW = 32 / NQ2;     // elements a warp
  static constexpr int LIVE = EPW * NQ2;   // lanes that hold nodes
};

template <int P, int RK>
__device__ __forceinline__ void col_load(ColIn<P>& in, const StageArgs& a, const ElemIndexer& idx,
                                         long long e, int c, int j, int k) {
  using C = ColShape<P>;
  constexpr int NQ = C::NQ;
  const ElemPos pos = idx.pos(e);
  const float* __restrict__ gu = static_cast<const float*>(a.u);
  const float* __restrict__ gv = static_cast<const float*>(a.v);
  const float* __restrict__ gw = static_cast<const float*>(a.w);
  const long long g = e * C::NP + NQ * c;
#pragma unroll
  for (int i = 0; i < NQ; i++) {
    in.q[i] = a.q_in[g + i];
    in.q0[i] = (RK == kRkGeneral) ? a.q0[g + i] : 0.0;
    in.u[i] = gu[g + i];
    in.v[i] = gv[g + i];
    in.w[i] = gw[g + i];
  }
  in.xm = face_gather<P, 0>(a, gu, pos, NQ * c, true);             // (0, j, k)
  in.xp = face_gather<P, 0>(a, gu, pos, NQ * c + NQ - 1, false);   // (NQ-1, j, k)
#pragma unroll
  for (int i = 0; i < NQ; i++) {
    in.y[i] = face_gather<P, 1>(a, gv, pos, NQ * c + i, j == 0, j == 0 || j == NQ - 1);
    in.z[i] = face_gather<P, 2>(a, gw, pos, NQ * c + i, k == 0, k == 0 || k == NQ - 1);
  }
}

template <int P, int RK>
__device__ __forceinline__ void col_compute(const ColIn<P>& in, const StageArgs& a, long long e,
                                            bool store, int s, int c, int j, int k,
                                            const float (&Tx)[EoShape<P>::TE],
                                            const WarpRow<P>& ry, const WarpRow<P>& rz) {
  using C = ColShape<P>;
  constexpr int NQ = C::NQ;
  float qf[NQ], acc[NQ];
#pragma unroll
  for (int i = 0; i < NQ; i++) qf[i] = to_ct<float>(in.q[i]);
  {  // x: the lane's own line, through eo_line_f as the block body runs it
    const float gm = face_flux(in.xm, true, qf[0], in.u[0]);
    const float gp = face_flux(in.xp, false, qf[NQ - 1], in.u[NQ - 1]);
    eo_line_f<P, 1, false, float>([&](int l) { return __fmul_rn(qf[l], in.u[l]); }, Tx, gm, gp,
                                  0, [&](int m, float v) { acc[m] = v; });
  }
  {  // y (face fluxes read from the lanes j = 0, NQ-1 only)
    float F[NQ], gf[NQ];
#pragma unroll
    for (int i = 0; i < NQ; i++) {
      F[i] = __fmul_rn(qf[i], in.v[i]);
      gf[i] = face_flux(in.y[i], j == 0, qf[i], in.v[i]);
    }
    const int base = C::NQ2 * s + NQ * k;
#pragma unroll
    for (int i = 0; i < NQ; i++) {
      float Fl[NQ];
#pragma unroll
      for (int l = 0; l < NQ; l++) Fl[l] = __shfl_sync(kFullMask, F[i], base + l);
      const float gm = __shfl_sync(kFullMask, gf[i], base);
      const float gp = __shfl_sync(kFullMask, gf[i], base + NQ - 1);
      acc[i] = acc[i] + ry.apply(Fl, gm, gp);
    }
  }
  {  // z (face fluxes from the lanes k = 0, NQ-1), then the RK update
    float F[NQ], gf[NQ];
#pragma unroll
    for (int i = 0; i < NQ; i++) {
      F[i] = __fmul_rn(qf[i], in.w[i]);
      gf[i] = face_flux(in.z[i], k == 0, qf[i], in.w[i]);
    }
    const int base = C::NQ2 * s + j;
    const long long g = e * C::NP + NQ * c;
#pragma unroll
    for (int i = 0; i < NQ; i++) {
      float Fl[NQ];
#pragma unroll
      for (int l = 0; l < NQ; l++) Fl[l] = __shfl_sync(kFullMask, F[i], base + NQ * l);
      const float gm = __shfl_sync(kFullMask, gf[i], base);
      const float gp = __shfl_sync(kFullMask, gf[i], base + NQ * (NQ - 1));
      const double inc = f32_to_f64_bits(acc[i] + rz.apply(Fl, gm, gp));
      if (!store) continue;
      if constexpr (RK == kRkTend)
        a.q_out[g + i] = inc;
      else
        a.q_out[g + i] = rk_combine<RK>(inc, in.q[i], in.q0[i], a.a, a.b);
    }
  }
}

template <int P, int RK>
__global__ void __launch_bounds__(WarpCfg<P>::THREADS, WarpCfg<P>::MIN_BLOCKS)
    stage_col_kernel(const StageArgs a) {
  using Sh = EoShape<P>;
  using C = ColShape<P>;
  const int lane = threadIdx.x & 31;
  const int ln = lane < C::LIVE ? lane : C::LIVE - 1;
  const int s = ln / C::NQ2, c = ln - C::NQ2 * s, j = c % C::NQ, k = c / C::NQ;
  const float* __restrict__ tab = static_cast<const float*>(a.D);
  float Tx[Sh::TE];  // the x direction's scaled tables, as the block body stages them
#pragma unroll
  for (int w = 0; w < Sh::TE; w++) Tx[w] = tab[w] * ((w < Sh::OFF_A) ? a.eo_sDf[0] : a.eo_sLf[0]);
  WarpRow<P> ry, rz;
  ry.load(tab, 1, a.eo_sDf[1], a.eo_sLf[1], j);
  rz.load(tab, 2, a.eo_sDf[2], a.eo_sLf[2], k);
  const long long end = a.elem_begin + a.elem_count;
  const ElemIndexer idx(a.box, end);
  constexpr int EPW = C::EPW;
  const long long step = (long long)EPW * gridDim.x * WarpCfg<P>::WARPS;
  // whole warps iterate together (the element set is warp-uniform), so every
  // lane takes part in the shuffles; a lane past the end works on the last
  // element and stores nothing
  long long e0 =
      a.elem_begin + (long long)EPW * ((long long)blockIdx.x * WarpCfg<P>::WARPS + (threadIdx.x >> 5));
  if (e0 >= end) return;
  auto elem = [&](long long b) { return b + s < end ? b + s : end - 1; };
  ColIn<P> cur;
  col_load<P, RK>(cur, a, idx, elem(e0), c, j, k);
  for (; e0 < end; e0 += step) {
    const bool store = lane < C::LIVE && e0 + s < end;
    if constexpr (WarpCfg<P>::PREFETCH) {
      ColIn<P> nxt;
      col_load<P, RK>(nxt, a, idx, elem(e0 + step < end ? e0 + step : e0), c, j, k);
      col_compute<P, RK>(cur, a, elem(e0), store, s, c, j, k, Tx, ry, rz);
      cur = nxt;
    } else {
      col_compute<P, RK>(cur, a, elem(e0), store, s, c, j, k, Tx, ry, rz);
      if (e0 + step < end) col_load<P, RK>(cur, a, idx, elem(e0 + step), c, j, k);
    }
  }
}

// p = 3: lane L holds nodes L and L + 32 (slot r), i.e. (i, j, k) = (L & 3,
// (L >> 2) & 3, (L >> 4) + 2 r).  The x and y lines of a node lie in its own
// slot; the z line of lane L is nodes (i, j, 0..3) = slot 0 of lanes L0 and
// L0 + 16, then slot 1 of the same lanes (L0 = L & 15), shared by the lane's
// two nodes (rows kh and 1 - kh, kh = L >> 4).  The - z face node of the line
// is slot 0 of lane L0 and the + z one slot 1 of lane L0 + 16, so every lane
// forms one z face flux.  p3_load issues all of an element's global loads
// together, as col_load does.
struct P3In {
  double q[2], q0[2];
  float u[2], v[2], w[2];
  FaceIn fx[2], fy[2], fz;
};

template <int RK>
__device__ __forceinline__ void p3_load(P3In& in, const StageArgs& a, const ElemIndexer& idx,
                                        long long e, int lane) {
  const int i = lane & 3, j = (lane >> 2) & 3, kh = lane >> 4;
  const float* __restrict__ gu = static_cast<const float*>(a.u);
  const float* __restrict__ gv = static_cast<const float*>(a.v);
  const float* __restrict__ gw = static_cast<const float*>(a.w);
  const ElemPos pos = idx.pos(e);
#pragma unroll
  for (int r = 0; r < 2; r++) {
    const long long g = e * 64 + lane + 32 * r;
    in.q[r] = a.q_in[g];
    in.q0[r] = (RK == kRkGeneral) ? a.q0[g] : 0.0;
    in.u[r] = gu[g];
    in.v[r] = gv[g];
    in.w[r] = gw[g];
    in.fx[r] = face_gather<3, 0>(a, gu, pos, lane + 32 * r, i == 0, i == 0 || i == 3);
    in.fy[r] = face_gather<3, 1>(a, gv, pos, lane + 32 * r, j == 0, j == 0 || j == 3);
  }
  in.fz = face_gather<3, 2>(a, gw, pos, kh == 0 ? lane : lane + 32, kh == 0);
}

template <int RK>
__device__ __forceinline__ void p3_compute(const P3In& in, const StageArgs& a, long long e,
                                           int lane, const WarpRow<3>& rx, const WarpRow<3>& ry,
                                           const WarpRow<3>& rz0, const WarpRow<3>& rz1) {
  constexpr int NQ = 4;
  const int i = lane & 3, j = (lane >> 2) & 3, kh = lane >> 4, L0 = lane & 15;
  const float qf0 = to_ct<float>(in.q[0]), qf1 = to_ct<float>(in.q[1]);
  float acc0, acc1;
  {  // x: each slot's own lines (face fluxes read from the lanes i = 0, 3 only)
    const float F0 = __fmul_rn(qf0, in.u[0]), F1 = __fmul_rn(qf1, in.u[1]);
    const float gf0 = face_flux(in.fx[0], i == 0, qf0, in.u[0]);
    const float gf1 = face_flux(in.fx[1], i == 0, qf1, in.u[1]);
    const int base = lane - i;
    float Fa[NQ], Fb[NQ];
#pragma unroll
    for (int c = 0; c < NQ; c++) {
      Fa[c] = __shfl_sync(kFullMask, F0, base + c);
      Fb[c] = __shfl_sync(kFullMask, F1, base + c);
    }
    acc0 = rx.apply(Fa, __shfl_sync(kFullMask, gf0, base),
                    __shfl_sync(kFullMask, gf0, base + NQ - 1));
    acc1 = rx.apply(Fb, __shfl_sync(kFullMask, gf1, base),
                    __shfl_sync(kFullMask, gf1, base + NQ - 1));
  }
  {  // y (face fluxes from the lanes j = 0, 3)
    const float F0 = __fmul_rn(qf0, in.v[0]), F1 = __fmul_rn(qf1, in.v[1]);
    const float gf0 = face_flux(in.fy[0], j == 0, qf0, in.v[0]);
    const float gf1 = face_flux(in.fy[1], j == 0, qf1, in.v[1]);
    const int base = lane - NQ * j;
    float Fa[NQ], Fb[NQ];
#pragma unroll
    for (int c = 0; c < NQ; c++) {
      Fa[c] = __shfl_sync(kFullMask, F0, base + NQ * c);
      Fb[c] = __shfl_sync(kFullMask, F1, base + NQ * c);
    }
    acc0 = acc0 + ry.apply(Fa, __shfl_sync(kFullMask, gf0, base),
                           __shfl_sync(kFullMask, gf0, base + NQ * (NQ - 1)));
    acc1 = acc1 + ry.apply(Fb, __shfl_sync(kFullMask, gf1, base),
                           __shfl_sync(kFullMask, gf1, base + NQ * (NQ - 1)));
  }
  float inc0, inc1;
  {  // z
    const float F0 = __fmul_rn(qf0, in.w[0]), F1 = __fmul_rn(qf1, in.w[1]);
    const bool minus = kh == 0;
    const float gf = face_flux(in.fz, minus, minus ? qf0 : qf1, minus ? in.w[0] : in.w[1]);
    float Fz[NQ];
    Fz[0] = __shfl_sync(kFullMask, F0, L0);
    Fz[1] = __shfl_sync(kFullMask, F0, L0 + 16);
    Fz[2] = __shfl_sync(kFullMask, F1, L0);
    Fz[3] = __shfl_sync(kFullMask, F1, L0 + 16);
    const float gm = __shfl_sync(kFullMask, gf, L0), gp = __shfl_sync(kFullMask, gf, L0 + 16);
    inc0 = acc0 + rz0.apply(Fz, gm, gp);
    inc1 = acc1 + rz1.apply(Fz, gm, gp);
  }
  const long long g0 = e * 64 + lane, g1 = g0 + 32;
  const double i0 = f32_to_f64_bits(inc0), i1 = f32_to_f64_bits(inc1);
  if constexpr (RK == kRkTend) {
    a.q_out[g0] = i0;
    a.q_out[g1] = i1;
  } else {
    a.q_out[g0] = rk_combine<RK>(i0, in.q[0], in.q0[0], a.a, a.b);
    a.q_out[g1] = rk_combine<RK>(i1, in.q[1], in.q0[1], a.a, a.b);
  }
}

template <int RK>
__global__ void __launch_bounds__(WarpCfg<3>::THREADS, WarpCfg<3>::MIN_BLOCKS)
    stage_p3_kernel(const StageArgs a) {
  constexpr int P = 3;
  const int lane = threadIdx.x & 31;
  const int i = lane & 3, j = (lane >> 2) & 3, kh = lane >> 4;
  const float* __restrict__ tab = static_cast<const float*>(a.D);
  WarpRow<P> rx, ry, rz0, rz1;
  rx.load(tab, 0, a.eo_sDf[0], a.eo_sLf[0], i);
  ry.load(tab, 1, a.eo_sDf[1], a.eo_sLf[1], j);
  rz0.load(tab, 2, a.eo_sDf[2], a.eo_sLf[2], kh);      // slot 0: k = kh
  rz1.load(tab, 2, a.eo_sDf[2], a.eo_sLf[2], 2 + kh);  // slot 1: k = 2 + kh
  const long long end = a.elem_begin + a.elem_count;
  const ElemIndexer idx(a.box, end);
  const long long step = (long long)gridDim.x * WarpCfg<P>::WARPS;
  long long e = a.elem_begin + (long long)blockIdx.x * WarpCfg<P>::WARPS + (threadIdx.x >> 5);
  if (e >= end) return;
  P3In cur;
  p3_load<RK>(cur, a, idx, e, lane);
  for (; e < end; e += step) {
    if constexpr (WarpCfg<P>::PREFETCH) {
      P3In nxt;
      p3_load<RK>(nxt, a, idx, e + step < end ? e + step : e, lane);
      p3_compute<RK>(cur, a, e, lane, rx, ry, rz0, rz1);
      cur = nxt;
    } else {
      p3_compute<RK>(cur, a, e, lane, rx, ry, rz0, rz1);
      if (e + step < end) p3_load<RK>(cur, a, idx, e + step, lane);
    }
  }
}

template <int P>
int launch_stage_warp_impl(const StageArgs& a, cudaStream_t st) {
  static_assert(P == 2 || P == 3, "warp-cooperative stage: p = 2 and 3");
  constexpr int T = WarpCfg<P>::THREADS, W = WarpCfg<P>::WARPS;
  constexpr int EPW = P == 2 ? ColShape<P>::EPW : 1;  // elements a warp at a time
  long long nblk = (a.elem_count + EPW * W - 1) / (EPW * W);
  if (nblk <= 0) return SDG_OK;
  // two waves of resident blocks, each warp striding over many elements: a
  // warp's set-up (its table rows, the index constants) is then paid once
  int dev = 0, nsm = 0;
  SDG_CUDA_TRY(cudaGetDevice(&dev));
  SDG_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const long long cap = 2LL * nsm * WarpCfg<P>::MIN_BLOCKS;
  if (nblk > cap) nblk = cap;
  const int kind = rk_kind(a);
  if constexpr (P == 2) {
    if (kind == kRkTend)
      stage_col_kernel<P, kRkTend><<<(unsigned)nblk, T, 0, st>>>(a);
    else if (kind == kRkFirst)
      stage_col_kernel<P, kRkFirst><<<(unsigned)nblk, T, 0, st>>>(a);
    else
      stage_col_kernel<P, kRkGeneral><<<(unsigned)nblk, T, 0, st>>>(a);
  } else {
    if (kind == kRkTend)
      stage_p3_kernel<kRkTend><<<(unsigned)nblk, T, 0, st>>>(a);
    else if (kind == kRkFirst)
      stage_p3_kernel<kRkFirst><<<(unsigned)nblk, T, 0, st>>>(a);
    else
      stage_p3_kernel<kRkGeneral><<<(unsigned)nblk, T, 0, st>>>(a);
  }
  SDG_CUDA_TRY(cudaGetLastError());
  return SDG_OK;
}

}  // namespace sdg
