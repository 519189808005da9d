// Element-per-thread form of the FP32-compute even-odd stage for the lowest
// order (p = 1; the generic form below also compiles for p = 2, where it
// measured level with the block body and is not used).
//
// At p = 1 an element has 8 nodes, 12 lines of two nodes and 24 face nodes:
// the block-cooperative body (stage_eo_block) spends most of its issue slots
// on distributing that little work -- per-task index division, face-node
// tables, shared-memory staging and four barriers -- and measured 82 % issue
// with DRAM at 20 % of its peak.  Here one thread owns a whole element for
// the whole stage: q, the velocity, the line results and the face fluxes of
// one direction at a time stay in registers, every index is a compile-time
// constant after unrolling, and there is no shared memory and no barrier.
// The neighbour gathers read the neighbour's face nodes straight from global
// memory (the x neighbour is the next thread's element, so most of them hit
// L1).
//
// The arithmetic is stage_eo_block<P, float>'s operation for operation --
// the same rounded products F = q u (__fmul_rn), the same five-operation face
// flux, eo_line_f's pair sums with the same scaled FP32 tables, the line
// results added in x, y, z order, the widened increment and the FP64 RK
// update -- so the result equals that body's bit for bit (tested), and the
// batched kernels, which keep the block body, stay bit-identical to the
// single-box solver.
#pragma once

#include "sdg_stage_eo.cuh"

namespace sdg {

template <int P>
struct ElemCfg {
  static constexpr int THREADS = 128;
  // resident blocks an SM the registers are capped for (64 and 128 a thread)
  static constexpr int MIN_BLOCKS = P == 1 ? 8 : 4;
};

// Node of position l on line r of direction D (x: r = j + NQ k, y: r = i +
// NQ k, z: r = i + NQ j), the line order of stage_eo_block.
template <int NQ, int D>
__device__ __forceinline__ constexpr int line_node(int r, int l) {
  return D == 0 ? l + NQ * r : D == 1 ? (r % NQ) + NQ * l + NQ * NQ * (r / NQ) : r + NQ * NQ * l;
}

// One direction D of one element: the face fluxes of the direction's - and
// + faces from the element's own values (qf, vel) and the neighbours' face
// values (qPm / uPm across the - face, qPp / uPp across the + face, in face
// node order fp = line r), then the lines: x results into acc, y results
// added, z results finished into the RK update (DEFER: z results only added
// into acc, the caller finishes the nodes).
template <int P, int D, int RK, bool DEFER = false>
__device__ __forceinline__ void elem_direction(const StageArgs& a, long long e,
                                               const float (&qf)[Ord<P>::NP],
                                               const float (&vel)[Ord<P>::NP],
                                               const float (&qPm)[Ord<P>::NFP],
                                               const float (&uPm)[Ord<P>::NFP],
                                               const float (&qPp)[Ord<P>::NFP],
                                               const float (&uPp)[Ord<P>::NFP], const float* T,
                                               float (&acc)[Ord<P>::NP]) {
  using O = Ord<P>;
  constexpr int NQ = O::NQ, NQ2 = O::NQ2, NP = O::NP, NFP = O::NFP;
  constexpr int FM = D == 0 ? 3 : D == 1 ? 0 : 4;  // the direction's - face
  constexpr int FPL = D == 0 ? 1 : D == 1 ? 2 : 5;  // and + face
  const double* __restrict__ qin = a.q_in;
  // face fluxes qP (±2 uP - |uP + uM|) - qM (±2 uM - |uP + uM|)
  float flm[NFP], flp[NFP];
#pragma unroll
  for (int side = 0; side < 2; side++) {
    const int f = side ? FPL : FM;
#pragma unroll
    for (int fp = 0; fp < NFP; fp++) {
      int nM, nP, axis, sg;
      face_nodes<NQ>(f, fp % NQ, fp / NQ, nM, nP, axis, sg);
      const float qM = qf[nM], uM = vel[nM];
      const float qP = side ? qPp[fp] : qPm[fp];
      const float uP = side ? uPp[fp] : uPm[fp];
      const float a2 = fabsf(uP + uM);
      const float tw = (sg > 0) ? 2.0f : -2.0f;
      const float tP = fmaf(tw, uP, -a2);
      const float tM = fmaf(tw, uM, -a2);
      (side ? flp : flm)[fp] = fmaf(qP, tP, -(qM * tM));
    }
  }
  const double rk_a = a.a, rk_b = a.b;
#pragma unroll
  for (int r = 0; r < NQ2; r++) {
    eo_line_f<P, 1, false, float>(
        [&](int l) { return __fmul_rn(qf[line_node<NQ, D>(r, l)], vel[line_node<NQ, D>(r, l)]); },
        T, flm[r], flp[r], 0, [&](int m, float v) {
          const int n = line_node<NQ, D>(r, m);
          if constexpr (D == 0) {
            acc[n] = v;
          } else if constexpr (D == 1 || DEFER) {
            acc[n] += v;
          } else {
            const long long g = e * NP + n;
            const double inc = f32_to_f64_bits(acc[n] + v);
            if constexpr (RK == kRkTend)
              a.q_out[g] = inc;
            else
              a.q_out[g] = rk_combine<RK>(inc, qin[g], RK == kRkGeneral ? a.q0[g] : 0.0, rk_a,
                                          rk_b);
          }
        });
  }
}

// The neighbours' face values of direction D gathered from global memory:
// for face f and face node fp, q (as FP32) and the axis velocity at the
// neighbour's opposite node.
template <int P, int D>
__device__ __forceinline__ void elem_gather(const double* __restrict__ qin,
                                            const float* __restrict__ gvel, const int (&nb)[6],
                                            float (&qPm)[Ord<P>::NFP], float (&uPm)[Ord<P>::NFP],
                                            float (&qPp)[Ord<P>::NFP], float (&uPp)[Ord<P>::NFP]) {
  using O = Ord<P>;
  constexpr int NQ = O::NQ, NP = O::NP, NFP = O::NFP;
  constexpr int FM = D == 0 ? 3 : D == 1 ? 0 : 4, FPL = D == 0 ? 1 : D == 1 ? 2 : 5;
#pragma unroll
  for (int side = 0; side < 2; side++) {
    const int f = side ? FPL : FM;
#pragma unroll
    for (int fp = 0; fp < NFP; fp++) {
      int nM, nP, axis, sg;
      face_nodes<NQ>(f, fp % NQ, fp / NQ, nM, nP, axis, sg);
      const long long gP = (long long)nb[f] * NP + nP;
      (side ? qPp : qPm)[fp] = to_ct<float>(qin[gP]);
      (side ? uPp : uPm)[fp] = gvel[gP];
    }
  }
}

template <int P, int RK>
__global__ void __launch_bounds__(ElemCfg<P>::THREADS, ElemCfg<P>::MIN_BLOCKS)
    stage_elem_kernel(const StageArgs a) {
  using O = Ord<P>;
  using Sh = EoShape<P>;
  constexpr int NP = O::NP, TE = Sh::TE;
  // the three directions' tables scaled as stage_eo_block stages them
  float T[3 * TE];
  const float* __restrict__ tab = static_cast<const float*>(a.D);
#pragma unroll
  for (int t = 0; t < 3 * TE; t++) {
    const int dir = t / TE, w = t - dir * TE;
    T[t] = tab[t] * ((w < Sh::OFF_A) ? a.eo_sDf[dir] : a.eo_sLf[dir]);
  }
  const float* __restrict__ gu = static_cast<const float*>(a.u);
  const float* __restrict__ gv = static_cast<const float*>(a.v);
  const float* __restrict__ gw = static_cast<const float*>(a.w);
  const long long end = a.elem_begin + a.elem_count;
  for (long long e = a.elem_begin + blockIdx.x * (long long)blockDim.x + threadIdx.x; e < end;
       e += (long long)gridDim.x * blockDim.x) {
    int nb[6];  // element indices are below 2^31 (checked at creation)
#pragma unroll
    for (int f = 0; f < 6; f++) nb[f] = (int)neighbor(a.box, e, f);
    float qf[NP], acc[NP], vel[NP];
    float qPm[Ord<P>::NFP], uPm[Ord<P>::NFP], qPp[Ord<P>::NFP], uPp[Ord<P>::NFP];
#pragma unroll
    for (int n = 0; n < NP; n++) qf[n] = to_ct<float>(a.q_in[e * NP + n]);
#pragma unroll
    for (int n = 0; n < NP; n++) vel[n] = gu[e * NP + n];
    elem_gather<P, 0>(a.q_in, gu, nb, qPm, uPm, qPp, uPp);
    elem_direction<P, 0, RK>(a, e, qf, vel, qPm, uPm, qPp, uPp, T, acc);
#pragma unroll
    for (int n = 0; n < NP; n++) vel[n] = gv[e * NP + n];
    elem_gather<P, 1>(a.q_in, gv, nb, qPm, uPm, qPp, uPp);
    elem_direction<P, 1, RK>(a, e, qf, vel, qPm, uPm, qPp, uPp, T + TE, acc);
#pragma unroll
    for (int n = 0; n < NP; n++) vel[n] = gw[e * NP + n];
    elem_gather<P, 2>(a.q_in, gw, nb, qPm, uPm, qPp, uPp);
    elem_direction<P, 2, RK>(a, e, qf, vel, qPm, uPm, qPp, uPp, T + 2 * TE, acc);

  }
}

// p = 1 with vector memory access: an element's 8 nodes are 64 contiguous
// bytes of q and 32 of each velocity component, so a thread loads them as
// 16-byte vectors; the y and z neighbours' face nodes are pairs or quads of
// adjacent nodes (16- and 32-byte vectors); the x neighbours are the elements
// of the adjacent lanes, whose face values arrive by warp shuffle (a global
// gather only at a warp edge or where the box wraps in x).  The node
// arithmetic is elem_direction's, so the bits are the block body's.
// Registers capped for four resident blocks of 128 threads (128 a thread, no
// spills): measured on GB300 at 128^3, 129.7 GDOF-updates/s against 123.1,
// 118.0 and 116.9 with the caps for five, six and eight blocks (which spill
// 16-150 bytes).
template <int RK>
__global__ void __launch_bounds__(128, 4) stage_p1_kernel(const StageArgs a) {
  using Sh = EoShape<1>;
  constexpr int TE = Sh::TE;
  float T[3 * TE];
  const float* __restrict__ tab = static_cast<const float*>(a.D);
#pragma unroll
  for (int t = 0; t < 3 * TE; t++) {
    const int dir = t / TE, w = t - dir * TE;
    T[t] = tab[t] * ((w < Sh::OFF_A) ? a.eo_sDf[dir] : a.eo_sLf[dir]);
  }
  const double2* __restrict__ q2 = reinterpret_cast<const double2*>(a.q_in);
  const double* __restrict__ qin = a.q_in;
  const float* __restrict__ gu = static_cast<const float*>(a.u);
  const float4* __restrict__ u4 = static_cast<const float4*>(a.u);
  const float2* __restrict__ v2 = static_cast<const float2*>(a.v);
  const float4* __restrict__ w4 = static_cast<const float4*>(a.w);
  const int lane = threadIdx.x & 31;
  const int NeX = a.box.NeX;
  const long long end = a.elem_begin + a.elem_count;
  const long long step = (long long)gridDim.x * blockDim.x;
  // whole warps iterate together, so every lane takes part in the shuffles
  for (long long wb = a.elem_begin + blockIdx.x * (long long)blockDim.x + (threadIdx.x & ~31);
       wb < end; wb += step) {
    const long long e0 = wb + lane;
    const bool valid = e0 < end;
    const long long e = valid ? e0 : end - 1;  // a safe element for idle lanes
    int nb[6];
#pragma unroll
    for (int f = 0; f < 6; f++) nb[f] = (int)neighbor(a.box, e, f);
    const int ex = (int)(e % NeX);
    float qf[8], vel[8], acc[8];
    double qd[8];
#pragma unroll
    for (int h = 0; h < 4; h++) {
      const double2 t = q2[e * 4 + h];
      qd[2 * h] = t.x;
      qd[2 * h + 1] = t.y;
    }
#pragma unroll
    for (int n = 0; n < 8; n++) qf[n] = to_ct<float>(qd[n]);
    float qPm[4], uPm[4], qPp[4], uPp[4];
    // x: u; the -x neighbour's i = 1 nodes (1, 3, 5, 7) from the lane below,
    // the +x neighbour's i = 0 nodes (0, 2, 4, 6) from the lane above
    {
      const float4 a0 = u4[e * 2], a1 = u4[e * 2 + 1];
      vel[0] = a0.x; vel[1] = a0.y; vel[2] = a0.z; vel[3] = a0.w;
      vel[4] = a1.x; vel[5] = a1.y; vel[6] = a1.z; vel[7] = a1.w;
      const bool from_lo = lane > 0 && ex > 0;
      const bool from_hi = lane < 31 && ex < NeX - 1 && e0 + 1 < end;
#pragma unroll
      for (int fp = 0; fp < 4; fp++) {
        const float qu = __shfl_up_sync(0xffffffffu, qf[2 * fp + 1], 1);
        const float uu = __shfl_up_sync(0xffffffffu, vel[2 * fp + 1], 1);
        const float qd_ = __shfl_down_sync(0xffffffffu, qf[2 * fp], 1);
        const float ud = __shfl_down_sync(0xffffffffu, vel[2 * fp], 1);
        qPm[fp] = qu;
        uPm[fp] = uu;
        qPp[fp] = qd_;
        uPp[fp] = ud;
      }
      if (!from_lo) {
#pragma unroll
        for (int fp = 0; fp < 4; fp++) {
          const long long g = (long long)nb[3] * 8 + 2 * fp + 1;
          qPm[fp] = to_ct<float>(qin[g]);
          uPm[fp] = gu[g];
        }
      }
      if (!from_hi) {
#pragma unroll
        for (int fp = 0; fp < 4; fp++) {
          const long long g = (long long)nb[1] * 8 + 2 * fp;
          qPp[fp] = to_ct<float>(qin[g]);
          uPp[fp] = gu[g];
        }
      }
    }
    elem_direction<1, 0, RK>(a, e, qf, vel, qPm, uPm, qPp, uPp, T, acc);
    // y: v; the -y neighbour's j = 1 nodes (2, 3, 6, 7), the +y
    // neighbour's j = 0 nodes (0, 1, 4, 5)
    {
#pragma unroll
      for (int h = 0; h < 4; h++) {
        const float2 t = v2[e * 4 + h];
        vel[2 * h] = t.x;
        vel[2 * h + 1] = t.y;
      }
      const long long bm = (long long)nb[0] * 4, bp = (long long)nb[2] * 4;
      const double2 m0 = q2[bm + 1], m1 = q2[bm + 3], p0 = q2[bp], p1 = q2[bp + 2];
      const float2 vm0 = v2[bm + 1], vm1 = v2[bm + 3], vp0 = v2[bp], vp1 = v2[bp + 2];
      qPm[0] = to_ct<float>(m0.x); qPm[1] = to_ct<float>(m0.y);
      qPm[2] = to_ct<float>(m1.x); qPm[3] = to_ct<float>(m1.y);
      uPm[0] = vm0.x; uPm[1] = vm0.y; uPm[2] = vm1.x; uPm[3] = vm1.y;
      qPp[0] = to_ct<float>(p0.x); qPp[1] = to_ct<float>(p0.y);
      qPp[2] = to_ct<float>(p1.x); qPp[3] = to_ct<float>(p1.y);
      uPp[0] = vp0.x; uPp[1] = vp0.y; uPp[2] = vp1.x; uPp[3] = vp1.y;
    }
    elem_direction<1, 1, RK>(a, e, qf, vel, qPm, uPm, qPp, uPp, T + TE, acc);
    // z: w; the -z neighbour's k = 1 nodes (4..7), the +z neighbour's k = 0
    // nodes (0..3)
    {
      const float4 a0 = w4[e * 2], a1 = w4[e * 2 + 1];
      vel[0] = a0.x; vel[1] = a0.y; vel[2] = a0.z; vel[3] = a0.w;
      vel[4] = a1.x; vel[5] = a1.y; vel[6] = a1.z; vel[7] = a1.w;
      const long long bm = (long long)nb[4] * 4, bp = (long long)nb[5] * 4;
      const double2 m0 = q2[bm + 2], m1 = q2[bm + 3], p0 = q2[bp], p1 = q2[bp + 1];
      const float4 wm = w4[(long long)nb[4] * 2 + 1], wp = w4[(long long)nb[5] * 2];
      qPm[0] = to_ct<float>(m0.x); qPm[1] = to_ct<float>(m0.y);
      qPm[2] = to_ct<float>(m1.x); qPm[3] = to_ct<float>(m1.y);
      uPm[0] = wm.x; uPm[1] = wm.y; uPm[2] = wm.z; uPm[3] = wm.w;
      qPp[0] = to_ct<float>(p0.x); qPp[1] = to_ct<float>(p0.y);
      qPp[2] = to_ct<float>(p1.x); qPp[3] = to_ct<float>(p1.y);
      uPp[0] = wp.x; uPp[1] = wp.y; uPp[2] = wp.z; uPp[3] = wp.w;
    }
    elem_direction<1, 2, RK, true>(a, e, qf, vel, qPm, uPm, qPp, uPp, T + 2 * TE, acc);
    if (!valid) continue;
    // finish: widened increments and the RK update, 16-byte stores
    double2* __restrict__ qo2 = reinterpret_cast<double2*>(a.q_out);
    const double2* __restrict__ q02 = reinterpret_cast<const double2*>(a.q0);
    const double ra = a.a, rb = a.b;
#pragma unroll
    for (int h = 0; h < 4; h++) {
      const double i0 = f32_to_f64_bits(acc[2 * h]), i1 = f32_to_f64_bits(acc[2 * h + 1]);
      double2 o;
      if constexpr (RK == kRkTend) {
        o = make_double2(i0, i1);
      } else if constexpr (RK == kRkFirst) {
        o = make_double2(rk_combine<RK>(i0, qd[2 * h], 0.0, ra, rb),
                         rk_combine<RK>(i1, qd[2 * h + 1], 0.0, ra, rb));
      } else {
        const double2 z = q02[e * 4 + h];
        o = make_double2(rk_combine<RK>(i0, qd[2 * h], z.x, ra, rb),
                         rk_combine<RK>(i1, qd[2 * h + 1], z.y, ra, rb));
      }
      qo2[e * 4 + h] = o;
    }
  }
}

template <int P>
int launch_stage_elem_impl(const StageArgs& a, cudaStream_t st) {
  constexpr int T = ElemCfg<P>::THREADS;
  long long nblk = (a.elem_count + T - 1) / T;
  if (nblk <= 0) return SDG_OK;
  if (nblk > 152LL * 64) nblk = 152LL * 64;  // grid-stride beyond 64 blocks an SM
  if constexpr (P == 1) {
    switch (rk_kind(a)) {
      case kRkTend: stage_p1_kernel<kRkTend><<<(unsigned)nblk, T, 0, st>>>(a); break;
      case kRkFirst: stage_p1_kernel<kRkFirst><<<(unsigned)nblk, T, 0, st>>>(a); break;
      default: stage_p1_kernel<kRkGeneral><<<(unsigned)nblk, T, 0, st>>>(a); break;
    }
    SDG_CUDA_TRY(cudaGetLastError());
    return SDG_OK;
  }
  switch (rk_kind(a)) {
    case kRkTend: stage_elem_kernel<P, kRkTend><<<(unsigned)nblk, T, 0, st>>>(a); break;
    case kRkFirst: stage_elem_kernel<P, kRkFirst><<<(unsigned)nblk, T, 0, st>>>(a); break;
    default: stage_elem_kernel<P, kRkGeneral><<<(unsigned)nblk, T, 0, st>>>(a); break;
  }
  SDG_CUDA_TRY(cudaGetLastError());
  return SDG_OK;
}

}  // namespace sdg
