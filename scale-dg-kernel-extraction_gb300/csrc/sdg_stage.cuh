// Fused RK-stage kernel for the periodic structured box.
//
// One launch advances every element of the box through one SSP-RK3 stage,
// replacing, per stage, the reference's update_halo (mod_mesh.f90:209-221),
// advect3d_eq_cal_tend (mod_advect3d_eq.f90:41-85: cal_elembnd_flux :89-142
// and cal_dqdt :146-201 with the DG operators of mod_dg_optr_kernel.f90) and
// the RK combine of main.f90:68-73.  A block owns EPB consecutive elements:
//
//   phase 0  D1D and the 6 neighbour elements of each element (periodic
//            wrap, computed once per element), and the block's nodes staged
//            in shared memory as q and F_d = q*u_d (coalesced loads);
//   phase 1  upwind flux on all 6*Nfp face nodes of each element: the minus
//            side's q from shared memory, its velocity and the plus side's q
//            and velocity from global memory (the neighbour's opposite face,
//            which is what VMapP plus the halo buffer encode);
//   phase 3  per node: sum-factorised Dx/Dy/Dz contractions, the lift of the
//            face fluxes, dqdt = -(Es_x Dx + Es_y Dy + Es_z Dz + Lift) and
//            q_out = a*q0 + b*(q + dt*dqdt).
//
// The stage reads q_in and q0 and writes q_out, three distinct buffers, so a
// block never overwrites what another block still gathers.
#pragma once

#include <cuda_runtime.h>

#include <type_traits>

#include "sdg_df.cuh"
#include "sdg_internal.h"

namespace sdg {

// RK update kinds of a stage, decided once per launch so that a node issues
// only its own FP64 operations: a per-node select between an add and an FMA
// would be if-converted into both, on the 1/64-rate FP64 pipe.
//   kRkTend     q_out = the tendency increment (c = 1, no state update)
//   kRkFirst    q_out = q + inc                 (b = 1, a = 0: stage 1)
//   kRkGeneral  q_out = a q0 + (b q + inc)
constexpr int kRkTend = 0, kRkFirst = 1, kRkGeneral = 2;

__host__ __device__ inline int rk_kind(const StageArgs& a) {
  return a.tend_only ? kRkTend : (a.b_is_one && !a.a_nonzero) ? kRkFirst : kRkGeneral;
}

template <int RK>
__device__ __forceinline__ double rk_combine(double inc, double qv, double q0v, double ra,
                                             double rb) {
  if constexpr (RK == kRkFirst)
    return qv + inc;
  else
    return fma(ra, q0v, fma(rb, qv, inc));
}

// Calls f(std::integral_constant<int, RK>{}) for the launch's RK kind.  A
// caller that knows the kind at compile time passes it as FIXED (>= 0), and
// only that variant is instantiated (the batched kernel, whose many order
// bodies would otherwise triple).
template <int FIXED = -1, typename F>
__device__ __forceinline__ void with_rk_kind(int kind, F&& f) {
  if constexpr (FIXED >= 0)
    f(std::integral_constant<int, FIXED>{});
  else if (kind == kRkTend)
    f(std::integral_constant<int, kRkTend>{});
  else if (kind == kRkFirst)
    f(std::integral_constant<int, kRkFirst>{});
  else
    f(std::integral_constant<int, kRkGeneral>{});
}

template <int P>
struct Ord {
  static constexpr int NQ = P + 1;
  static constexpr int NQ2 = NQ * NQ;
  static constexpr int NP = NQ * NQ2;
  static constexpr int NFP = NQ2;
  static constexpr int NFT = 6 * NFP;
};

// Elements per block and threads per block of the fused stage kernel.
template <int P, typename CT>
struct StageCfg {
  static constexpr int EPB = (P == 1) ? 32 : (P == 2) ? 16 : (P == 3) ? 8
                           : (P == 4) ? 4 : (P <= 6) ? 2 : 1;
  static constexpr int THREADS = (P >= 10) ? 512 : 256;
};

// sum_l Dcol[l*DS] * f[l*stride], l = 0..NQ-1.  GENERAL order: running sum
// from zero (mod_dg_optr_kernel.f90:216-256).  OPT1 for p > 7: three partial
// sums of round(NQ/3), round(NQ/3) and the rest, added as (t1+t2)+t3
// (mod_dg_optr_kernel_opt1.F90.erb:42-44, :257-273).  DS is the stride of the
// matrix entries: NQ for a row of D1D(i,:), 1 for a column of D1D_tr(:,j).
template <int NQ, bool SPLIT3, int DS, typename T>
__device__ __forceinline__ T line_sum(const T* __restrict__ Dcol,
                                      const T* __restrict__ f, int stride) {
  if constexpr (!SPLIT3) {
    T s = Dcol[0] * f[0];
#pragma unroll
    for (int l = 1; l < NQ; l++) s = fma(Dcol[l * DS], f[l * stride], s);
    return s;
  } else {
    constexpr int D3 = (2 * NQ + 3) / 6;  // round(NQ/3.0) for NQ in 9..16
    T t1 = Dcol[0] * f[0];
#pragma unroll
    for (int l = 1; l < D3; l++) t1 = fma(Dcol[l * DS], f[l * stride], t1);
    T t2 = Dcol[D3 * DS] * f[D3 * stride];
#pragma unroll
    for (int l = D3 + 1; l < 2 * D3; l++) t2 = fma(Dcol[l * DS], f[l * stride], t2);
    T t3 = Dcol[2 * D3 * DS] * f[2 * D3 * stride];
#pragma unroll
    for (int l = 2 * D3 + 1; l < NQ; l++) t3 = fma(Dcol[l * DS], f[l * stride], t3);
    return (t1 + t2) + t3;
  }
}

// Lift of one node (mod_dg_optr_kernel.f90:274-286), faces in order 1..6.
// L points at Lift_mat(n,1) (face stride NP); fl at the element's 6*NFP fluxes.
template <int P, typename T>
__device__ __forceinline__ T lift_node(const T* __restrict__ L,
                                       const T* __restrict__ fl, int i, int j,
                                       int k) {
  using O = Ord<P>;
  T s = __ldg(L) * fl[i + k * O::NQ];
  s = fma(__ldg(L + 1 * O::NP), fl[1 * O::NFP + j + k * O::NQ], s);
  s = fma(__ldg(L + 2 * O::NP), fl[2 * O::NFP + i + k * O::NQ], s);
  s = fma(__ldg(L + 3 * O::NP), fl[3 * O::NFP + j + k * O::NQ], s);
  s = fma(__ldg(L + 4 * O::NP), fl[4 * O::NFP + i + j * O::NQ], s);
  s = fma(__ldg(L + 5 * O::NP), fl[5 * O::NFP + i + j * O::NQ], s);
  return s;
}

// Face geometry of the structured element (mod_mesh.f90:265-324, :356-397):
// for face f (0-based: -y,+x,+y,-x,-z,+z) and tangential indices (ta, tb),
// the node on this face, the node with the same tangential indices on the
// opposite face, the normal axis and sign.
template <int NQ>
__device__ __forceinline__ void face_nodes(int f, int ta, int tb, int& nM,
                                           int& nP, int& axis, int& sgn) {
  constexpr int NQ2 = NQ * NQ, L = NQ - 1;
  switch (f) {
    case 0: nM = ta + tb * NQ2;              nP = ta + L * NQ + tb * NQ2;  axis = 1; sgn = -1; break;
    case 1: nM = L + ta * NQ + tb * NQ2;     nP = ta * NQ + tb * NQ2;      axis = 0; sgn = 1;  break;
    case 2: nM = ta + L * NQ + tb * NQ2;     nP = ta + tb * NQ2;           axis = 1; sgn = 1;  break;
    case 3: nM = ta * NQ + tb * NQ2;         nP = L + ta * NQ + tb * NQ2;  axis = 0; sgn = -1; break;
    case 4: nM = ta + tb * NQ;               nP = ta + tb * NQ + L * NQ2;  axis = 2; sgn = -1; break;
    default: nM = ta + tb * NQ + L * NQ2;    nP = ta + tb * NQ;            axis = 2; sgn = 1;  break;
  }
}

// Face-flux task t (t < nloc * 6 Nq^2) of a block with nloc elements ->
// element le, face f, face node fp.  Below p = 5 a face has fewer nodes than
// a warp has lanes, and tasks taken element by element mix two to four faces
// in a warp, each lane on its own branch of face_nodes; there the tasks go
// face-major (every element's nodes of face 0, then face 1, ...), which keeps
// the face uniform across a warp but at face boundaries.  The face is found
// by a multiply-high with ceil(2^32 / W), W = nloc Nq^2, exact for t W < 2^32.
// The task's element-major index le * 6 Nq^2 + f Nq^2 + fp is what the face
// arrays are indexed by in either order.
template <int NQ>
struct FaceTasks {
  static constexpr int NFP = NQ * NQ, NFT = 6 * NFP;
  unsigned W, magic;
  __device__ __forceinline__ explicit FaceTasks(int nloc)
      : W((unsigned)(nloc * NFP)), magic(0xFFFFFFFFu / (unsigned)(nloc * NFP) + 1u) {}
  __device__ __forceinline__ void map(int t, int& le, int& f, int& fp) const {
    if constexpr (NFP < 32) {
      f = (int)__umulhi((unsigned)t, magic);
      const int rem = t - f * (int)W;
      le = rem / NFP;
      fp = rem - le * NFP;
    } else {
      le = t / NFT;
      const int r = t - le * NFT;
      f = r / NFP;
      fp = r - f * NFP;
    }
  }
};

// Neighbour across face f with periodic wrap (eval_neighbor_element,
// mod_mesh.f90:407-483); element index e = ex + ey*NeX + ez*NeX*NeY.  The
// element count is below 2^31 (checked at creation), so the index arithmetic
// is 32-bit: 64-bit division is a long software sequence on the GPU.
__device__ __forceinline__ long long neighbor(const Box& b, long long e64, int f) {
  const int NeX = b.NeX, NeY = b.NeY, NeZ = b.NeZ;
  const unsigned e = (unsigned)e64;
  const unsigned rxy = e / (unsigned)NeX;
  int ex = (int)(e - rxy * (unsigned)NeX);
  const unsigned rz = rxy / (unsigned)NeY;
  int ey = (int)(rxy - rz * (unsigned)NeY);
  int ez = (int)rz;
  switch (f) {
    case 0: ey = (ey == 0) ? NeY - 1 : ey - 1; break;
    case 1: ex = (ex == NeX - 1) ? 0 : ex + 1; break;
    case 2: ey = (ey == NeY - 1) ? 0 : ey + 1; break;
    case 3: ex = (ex == 0) ? NeX - 1 : ex - 1; break;
    case 4: ez = (ez == 0) ? NeZ - 1 : ez - 1; break;
    default: ez = (ez == NeZ - 1) ? 0 : ez + 1; break;
  }
  return (long long)((unsigned)ex + (unsigned)NeX * ((unsigned)ey + (unsigned)NeY * (unsigned)ez));
}

// Conversions into the compute type.  FP64 -> FP32 goes through the bit
// pattern (df_split's high part: 24 significant bits, round half up on the
// magnitude, |x| < 2^-126 flushed to zero) because the F2F conversion runs on
// GB300's FP64 pipe at 1/64 of the FP32 rate.
template <typename T> __device__ __forceinline__ T to_ct(double x) { return (T)x; }
template <> __device__ __forceinline__ float to_ct<float>(double x) { return df_split(x).hi; }
template <typename T> __device__ __forceinline__ T to_ct(float x) { return (T)x; }


// Dynamic shared memory of one block holding `nloc` elements of order P:
// D1D, then per element q, F_x, F_y, F_z (Np each) and the face fluxes (6 Nfp),
// then the 6 neighbour indices of every element.
template <int P, typename CT>
__host__ __device__ constexpr size_t stage_block_smem(int nloc) {
  using O = Ord<P>;
  return sizeof(CT) * (size_t)(O::NQ2 + nloc * (4 * O::NP + O::NFT)) + sizeof(int) * 6 * nloc;
}

// One block advances elements [eb, eb + nloc) of the box in `a` through one
// stage.  The block size and nloc are runtime values, so the batched
// persistent kernel can run any order and any elements-per-block choice
// through the same body; `smem` holds stage_block_smem<P, CT>(nloc) bytes.
template <int P, typename CT, typename VT, bool SPLIT3, int RKFIX = -1>
__device__ __forceinline__ void stage_block(const StageArgs& a, long long eb, int nloc,
                                            unsigned char* smem) {
  using O = Ord<P>;
  constexpr int NQ = O::NQ, NQ2 = O::NQ2, NP = O::NP, NFP = O::NFP, NFT = O::NFT;
  const int T = blockDim.x;
  CT* sD = reinterpret_cast<CT*>(smem);
  CT* sq = sD + NQ2;
  CT* su = sq + nloc * NP;  // F_x after phase 0
  CT* sv = su + nloc * NP;  // F_y
  CT* sw = sv + nloc * NP;  // F_z
  CT* sf = sw + nloc * NP;
  int* snb = reinterpret_cast<int*>(sf + nloc * NFT);

  const double* __restrict__ qin = a.q_in;
  const VT* __restrict__ gu = static_cast<const VT*>(a.u);
  const VT* __restrict__ gv = static_cast<const VT*>(a.v);
  const VT* __restrict__ gw = static_cast<const VT*>(a.w);
  const long long g0 = eb * NP;

  // phase 0: D1D, neighbour elements (once per element, not per face node),
  // and the staged state with the volume fluxes F_d = q * u_d
  // (mod_advect3d_eq.f90:181-183)
  for (int t = threadIdx.x; t < NQ2; t += T) sD[t] = static_cast<const CT*>(a.D)[t];
  for (int t = threadIdx.x; t < 6 * nloc; t += T)
    snb[t] = (int)neighbor(a.box, eb + t / 6, t % 6);
  for (int t = threadIdx.x; t < nloc * NP; t += T) {
    const CT qq = to_ct<CT>(qin[g0 + t]);
    sq[t] = qq;
    su[t] = qq * to_ct<CT>(gu[g0 + t]);
    sv[t] = qq * to_ct<CT>(gv[g0 + t]);
    sw[t] = qq * to_ct<CT>(gw[g0 + t]);
  }
  __syncthreads();

  // phase 1: element-boundary flux (mod_advect3d_eq.f90:116-140); 0.5*Fscale
  // is exact in either type and prepared on the host for FP32.  The velocity
  // of both sides is read from global memory (the own element's values were
  // just loaded by phase 0 and sit in L1).
  CT hfx, hfy, hfz;
  if constexpr (sizeof(CT) == 4) {
    hfx = a.box.hFsf[0];
    hfy = a.box.hFsf[1];
    hfz = a.box.hFsf[2];
  } else {
    hfx = 0.5 * a.box.Fs[0];
    hfy = 0.5 * a.box.Fs[1];
    hfz = 0.5 * a.box.Fs[2];
  }
  const FaceTasks<NQ> ftask(nloc);
  for (int t = threadIdx.x; t < nloc * NFT; t += T) {
    int le, f, fp;
    ftask.map(t, le, f, fp);
    const int r = f * NFP + fp;
    int nM, nP, axis, sg;
    face_nodes<NQ>(f, fp % NQ, fp / NQ, nM, nP, axis, sg);
    const long long gM = g0 + (long long)le * NP + nM;
    const long long gP = (long long)snb[6 * le + f] * NP + nP;
    const VT* gvel = (axis == 0) ? gu : (axis == 1) ? gv : gw;
    // normal velocity u.n with an axis-aligned unit normal is +-u_axis
    // exactly; the sign is applied by negation, not by a multiply
    const CT uM = to_ct<CT>(gvel[gM]), uP = to_ct<CT>(gvel[gP]);
    const CT velM = (sg > 0) ? uM : -uM;
    const CT velP = (sg > 0) ? uP : -uP;
    const CT qM = sq[le * NP + nM];
    const CT qP = to_ct<CT>(qin[gP]);
    const CT alpha = CT(0.5) * fabs(velP + velM);
    const CT hfs = (axis == 0) ? hfx : (axis == 1) ? hfy : hfz;
    sf[le * NFT + r] = hfs * ((qP * velP - qM * velM) - alpha * (qP - qM));
  }
  __syncthreads();

  // phase 3: divergence + lift + combine + RK (mod_advect3d_eq.f90:185-198,
  // main.f90:69-73)
  CT Ex, Ey, Ez;
  if constexpr (sizeof(CT) == 4) {
    Ex = a.box.Esf[0];
    Ey = a.box.Esf[1];
    Ez = a.box.Esf[2];
  } else {
    Ex = a.box.Es[0];
    Ey = a.box.Es[1];
    Ez = a.box.Es[2];
  }
  const CT* __restrict__ L = static_cast<const CT*>(a.Lift);
  double* __restrict__ qout = a.q_out;
  const double* __restrict__ q0 = a.q0;
  const double ra = a.a, rb = a.b, rdt = a.dt;
  const CT cdt = a.cdt_hi;
  with_rk_kind<RKFIX>(rk_kind(a), [&](auto rkc) {
    constexpr int RK = decltype(rkc)::value;
    for (int t = threadIdx.x; t < nloc * NP; t += T) {
      const int le = t / NP;
      const int n = t - le * NP;
      const int i = n % NQ;
      const int j = (n / NQ) % NQ;
      const int k = n / NQ2;
      const CT* Fx = su + le * NP;
      const CT* Fy = sv + le * NP;
      const CT* Fz = sw + le * NP;
      const CT dx = line_sum<NQ, SPLIT3, NQ>(sD + i, Fx + j * NQ + k * NQ2, 1);
      const CT dy = line_sum<NQ, SPLIT3, NQ>(sD + j, Fy + i + k * NQ2, NQ);
      const CT dz = line_sum<NQ, SPLIT3, NQ>(sD + k, Fz + i + j * NQ, NQ2);
      const CT lf = lift_node<P>(L + n, sf + le * NFT, i, j, k);
      const CT dq = -(((Ex * dx + Ey * dy) + Ez * dz) + lf);
      const long long g = g0 + t;
      if constexpr (sizeof(CT) == 8) {
        // the reference's order, a*q0 + b*(q + dt*dqdt) (main.f90:69-73);
        // stage 1 (a = 0, b = 1) is q + dt*dqdt exactly
        if constexpr (RK == kRkTend) {
          qout[g] = (double)dq;
        } else if constexpr (RK == kRkFirst) {
          qout[g] = qin[g] + rdt * (double)dq;
        } else {
          const double r = rb * (qin[g] + rdt * (double)dq);
          qout[g] = ra * q0[g] + r;
        }
      } else {
        // FP32 form: the increment (b*dt)*dqdt is an FP32 product widened by
        // bits; the state combination a*q0 + b*q + increment stays FP64
        if constexpr (RK == kRkTend)
          qout[g] = f32_to_f64_bits(dq);
        else
          qout[g] = rk_combine<RK>(f32_to_f64_bits(cdt * dq), qin[g],
                                   RK == kRkGeneral ? q0[g] : 0.0, ra, rb);
      }
    }
  });
}

template <int P, typename CT, typename VT, bool SPLIT3>
constexpr size_t stage_smem_bytes() {
  return stage_block_smem<P, CT>(StageCfg<P, CT>::EPB);
}

template <int P, typename CT, typename VT, bool SPLIT3>
__global__ void __launch_bounds__(StageCfg<P, CT>::THREADS)
    stage_kernel(const StageArgs a) {
  constexpr int EPB = StageCfg<P, CT>::EPB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const long long eb = a.elem_begin + (long long)blockIdx.x * EPB;
  const long long eend = a.elem_begin + a.elem_count;
  const int nloc = (int)((eend - eb) < EPB ? (eend - eb) : EPB);
  if (nloc <= 0) return;
  stage_block<P, CT, VT, SPLIT3>(a, eb, nloc, smem_raw);
}

template <int P, typename CT, typename VT, bool SPLIT3>
int launch_stage_impl(const StageArgs& a, cudaStream_t st) {
  using C = StageCfg<P, CT>;
  constexpr size_t smem = stage_smem_bytes<P, CT, VT, SPLIT3>();
  SDG_TRY(set_kernel_smem((const void*)stage_kernel<P, CT, VT, SPLIT3>, (int)smem, false));
  const long long nblk = (a.elem_count + C::EPB - 1) / C::EPB;
  if (nblk <= 0) return SDG_OK;
  if (nblk > 0x7fffffffLL) return fail(SDG_ERR_INVALID_ARG, "too many elements");
  stage_kernel<P, CT, VT, SPLIT3><<<(unsigned)nblk, C::THREADS, smem, st>>>(a);
  SDG_CUDA_TRY(cudaGetLastError());
  return SDG_OK;
}

}  // namespace sdg
