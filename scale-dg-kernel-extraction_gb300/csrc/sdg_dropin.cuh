// Kernels behind the reference-shaped entry points, for meshes given as the
// reference's arrays (VMapM/VMapP with a halo buffer, normal_fn, Escale,
// Fscale), so any connectivity the caller builds is honoured.
//
//   flux_kernel      cal_elembnd_flux (mod_advect3d_eq.f90:89-142), one
//                    thread per face node, VMap indices range-checked;
//   dqdt_kernel      cal_dqdt (mod_advect3d_eq.f90:146-201), EPB elements
//                    per block staged in shared memory;
//   divlike_kernel   tensorprod_divlike_dirXYZ (mod_dg_optr_kernel.f90:62-136)
//                    over a batch of elements;
//   lift_kernel      tensorprod_Lift_hexahedral (mod_dg_optr_kernel.f90:139-190).
#pragma once

#include "sdg_stage.cuh"

namespace sdg {

struct TendArgs {
  double* dqdt;
  const double* q;
  const double* u;
  const double* v;
  const double* w;
  const double* D;      // D1D(Nq,Nq)
  const double* Dt;     // D1D_tr(Nq,Nq)
  const double* Lift;   // Lift_mat(Nq,Nq,Nq,6)
  const int* VMapM;
  const int* VMapP;
  const double* normal_fn;
  const double* Escale;
  const double* Fscale;
  double* flux;         // ebnd_flux(NfpTot,Ne)
  int* err;             // set to 1 on an out-of-range VMap entry
  int Ne;
  long long NpNeA;      // Np*NeA: valid 1-based indices are 1..NpNeA
};

template <int P>
struct DropCfg {
  static constexpr int EPB = (P <= 2) ? 8 : (P <= 4) ? 2 : 1;
  static constexpr int THREADS = (P >= 10) ? 512 : 256;
};

template <int P>
constexpr size_t dqdt_smem_bytes() {
  using O = Ord<P>;
  return sizeof(double) * (size_t)(2 * O::NQ2 + DropCfg<P>::EPB * 3 * O::NP);
}

// cal_dqdt for elements [blockIdx.x*EPB, ...): F_d = q*u_d, divergence with
// D1D (x) and D1D_tr (y, z) exactly as tensorprod_divlike_dirXYZ reads them,
// lift of flux(:,ke), combine with Escale(:,ke,d).
template <int P, bool SPLIT3>
__global__ void __launch_bounds__(DropCfg<P>::THREADS) dqdt_kernel(const TendArgs a) {
  using O = Ord<P>;
  constexpr int NQ = O::NQ, NQ2 = O::NQ2, NP = O::NP, NFT = O::NFT,
                EPB = DropCfg<P>::EPB, T = DropCfg<P>::THREADS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* sD = reinterpret_cast<double*>(smem_raw);
  double* sDt = sD + NQ2;
  double* fx = sDt + NQ2;
  double* fy = fx + EPB * NP;
  double* fz = fy + EPB * NP;
  const long long eb = (long long)blockIdx.x * EPB;
  const int nloc = (int)min((long long)EPB, (long long)a.Ne - eb);
  if (nloc <= 0) return;
  for (int t = threadIdx.x; t < NQ2; t += T) {
    sD[t] = a.D[t];
    sDt[t] = a.Dt[t];
  }
  const long long g0 = eb * NP;
  for (int t = threadIdx.x; t < nloc * NP; t += T) {
    const double qq = a.q[g0 + t];
    fx[t] = qq * a.u[g0 + t];
    fy[t] = qq * a.v[g0 + t];
    fz[t] = qq * a.w[g0 + t];
  }
  __syncthreads();
  const long long NpNe = (long long)NP * a.Ne;
  for (int t = threadIdx.x; t < nloc * NP; t += T) {
    const int le = t / NP;
    const int n = t - le * NP;
    const int i = n % NQ, j = (n / NQ) % NQ, k = n / NQ2;
    const double dx = line_sum<NQ, SPLIT3, NQ>(sD + i, fx + le * NP + j * NQ + k * NQ2, 1);
    const double dy = line_sum<NQ, SPLIT3, 1>(sDt + j * NQ, fy + le * NP + i + k * NQ2, NQ);
    const double dz = line_sum<NQ, SPLIT3, 1>(sDt + k * NQ, fz + le * NP + i + j * NQ, NQ2);
    const double lf = lift_node<P>(a.Lift + n, a.flux + (eb + le) * NFT, i, j, k);
    const long long g = g0 + t;
    a.dqdt[g] = -(((a.Escale[g] * dx + a.Escale[g + NpNe] * dy) +
                   a.Escale[g + 2 * NpNe] * dz) + lf);
  }
}

struct DivArgs {
  double* ox;
  double* oy;
  double* oz;
  const double* D;
  const double* Dt;
  const double* ix;
  const double* iy;
  const double* iz;
  int nelem;
};

template <int P>
constexpr size_t divlike_smem_bytes() {
  using O = Ord<P>;
  return sizeof(double) * (size_t)(2 * O::NQ2 + DropCfg<P>::EPB * 3 * O::NP);
}

template <int P, bool SPLIT3>
__global__ void __launch_bounds__(DropCfg<P>::THREADS) divlike_kernel(const DivArgs a) {
  using O = Ord<P>;
  constexpr int NQ = O::NQ, NQ2 = O::NQ2, NP = O::NP, EPB = DropCfg<P>::EPB,
                T = DropCfg<P>::THREADS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* sD = reinterpret_cast<double*>(smem_raw);
  double* sDt = sD + NQ2;
  double* fx = sDt + NQ2;
  double* fy = fx + EPB * NP;
  double* fz = fy + EPB * NP;
  const long long eb = (long long)blockIdx.x * EPB;
  const int nloc = (int)min((long long)EPB, (long long)a.nelem - eb);
  if (nloc <= 0) return;
  for (int t = threadIdx.x; t < NQ2; t += T) {
    sD[t] = a.D[t];
    sDt[t] = a.Dt[t];
  }
  const long long g0 = eb * NP;
  for (int t = threadIdx.x; t < nloc * NP; t += T) {
    fx[t] = a.ix[g0 + t];
    fy[t] = a.iy[g0 + t];
    fz[t] = a.iz[g0 + t];
  }
  __syncthreads();
  for (int t = threadIdx.x; t < nloc * NP; t += T) {
    const int le = t / NP;
    const int n = t - le * NP;
    const int i = n % NQ, j = (n / NQ) % NQ, k = n / NQ2;
    a.ox[g0 + t] = line_sum<NQ, SPLIT3, NQ>(sD + i, fx + le * NP + j * NQ + k * NQ2, 1);
    a.oy[g0 + t] = line_sum<NQ, SPLIT3, 1>(sDt + j * NQ, fy + le * NP + i + k * NQ2, NQ);
    a.oz[g0 + t] = line_sum<NQ, SPLIT3, 1>(sDt + k * NQ, fz + le * NP + i + j * NQ, NQ2);
  }
}

template <int P>
__global__ void lift_kernel(double* out, const double* Lift, const double* in,
                            int nelem) {
  using O = Ord<P>;
  const long long total = (long long)O::NP * nelem;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    const long long e = g / O::NP;
    const int n = (int)(g - e * O::NP);
    const int i = n % O::NQ, j = (n / O::NQ) % O::NQ, k = n / O::NQ2;
    out[g] = lift_node<P>(Lift + n, in + e * O::NFT, i, j, k);
  }
}

template <int P, bool SPLIT3>
int launch_dqdt_impl(const TendArgs& a, cudaStream_t st) {
  constexpr size_t smem = dqdt_smem_bytes<P>();
  SDG_CUDA_TRY(cudaFuncSetAttribute(dqdt_kernel<P, SPLIT3>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
  const long long nblk = ((long long)a.Ne + DropCfg<P>::EPB - 1) / DropCfg<P>::EPB;
  if (nblk == 0) return SDG_OK;
  dqdt_kernel<P, SPLIT3><<<(unsigned)nblk, DropCfg<P>::THREADS, smem, st>>>(a);
  SDG_CUDA_TRY(cudaGetLastError());
  return SDG_OK;
}

// element_operation_kernel_matvec_gradlike_dirXYZ_P* (erb:166-219): the
// three directional contractions of ONE field (a.ix; a.iy and a.iz unused),
// always as a running sum over l (the template has no three-way split).  The
// z direction contracts along k, Σ_l vec_in(i,j,l) Mat_tr(l,k); the
// template's first z term, vec_in(i,1,k)*Mat_tr(1,j), is a typo and is not
// reproduced.  The field is staged once per element, so a DOF costs one read
// and three writes.  A NULL output is skipped: with one output this is the
// single-direction matvec_dirX / dirY / dirZ (erb:51-129).
template <int P>
constexpr size_t gradlike_smem_bytes() {
  using O = Ord<P>;
  return sizeof(double) * (size_t)(2 * O::NQ2 + DropCfg<P>::EPB * O::NP);
}

template <int P>
__global__ void __launch_bounds__(DropCfg<P>::THREADS) gradlike_kernel(const DivArgs a) {
  using O = Ord<P>;
  constexpr int NQ = O::NQ, NQ2 = O::NQ2, NP = O::NP, EPB = DropCfg<P>::EPB,
                T = DropCfg<P>::THREADS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* sD = reinterpret_cast<double*>(smem_raw);
  double* sDt = sD + NQ2;
  double* f = sDt + NQ2;
  const long long eb = (long long)blockIdx.x * EPB;
  const int nloc = (int)min((long long)EPB, (long long)a.nelem - eb);
  if (nloc <= 0) return;
  for (int t = threadIdx.x; t < NQ2; t += T) {
    sD[t] = a.D[t];
    sDt[t] = a.Dt[t];
  }
  const long long g0 = eb * NP;
  for (int t = threadIdx.x; t < nloc * NP; t += T) f[t] = a.ix[g0 + t];
  __syncthreads();
  for (int t = threadIdx.x; t < nloc * NP; t += T) {
    const int le = t / NP;
    const int n = t - le * NP;
    const int i = n % NQ, j = (n / NQ) % NQ, k = n / NQ2;
    const double* fe = f + le * NP;
    if (a.ox) a.ox[g0 + t] = line_sum<NQ, false, NQ>(sD + i, fe + j * NQ + k * NQ2, 1);
    if (a.oy) a.oy[g0 + t] = line_sum<NQ, false, 1>(sDt + j * NQ, fe + i + k * NQ2, NQ);
    if (a.oz) a.oz[g0 + t] = line_sum<NQ, false, 1>(sDt + k * NQ, fe + i + j * NQ, NQ2);
  }
}

template <int P>
int launch_gradlike_impl(const DivArgs& a, cudaStream_t st) {
  constexpr size_t smem = gradlike_smem_bytes<P>();
  SDG_CUDA_TRY(cudaFuncSetAttribute(gradlike_kernel<P>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const long long nblk = ((long long)a.nelem + DropCfg<P>::EPB - 1) / DropCfg<P>::EPB;
  if (nblk == 0) return SDG_OK;
  gradlike_kernel<P><<<(unsigned)nblk, DropCfg<P>::THREADS, smem, st>>>(a);
  SDG_CUDA_TRY(cudaGetLastError());
  return SDG_OK;
}

template <int P, bool SPLIT3>
int launch_divlike_impl(const DivArgs& a, cudaStream_t st) {
  constexpr size_t smem = divlike_smem_bytes<P>();
  SDG_CUDA_TRY(cudaFuncSetAttribute(divlike_kernel<P, SPLIT3>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
  const long long nblk = ((long long)a.nelem + DropCfg<P>::EPB - 1) / DropCfg<P>::EPB;
  if (nblk == 0) return SDG_OK;
  divlike_kernel<P, SPLIT3><<<(unsigned)nblk, DropCfg<P>::THREADS, smem, st>>>(a);
  SDG_CUDA_TRY(cudaGetLastError());
  return SDG_OK;
}

template <int P>
int launch_lift_impl(double* out, const double* Lift, const double* in, int nelem,
                     cudaStream_t st) {
  const long long total = (long long)Ord<P>::NP * nelem;
  if (total == 0) return SDG_OK;
  const long long nb = (total + 255) / 256;
  lift_kernel<P><<<(unsigned)(nb < 65535LL * 32 ? nb : 65535LL * 32), 256, 0, st>>>(
      out, Lift, in, nelem);
  SDG_CUDA_TRY(cudaGetLastError());
  return SDG_OK;
}

// Per-order entry used by the dispatch in sdg_dropin.cu.
template <int P>
int dropin_order(int what, int opt, const void* args, cudaStream_t st) {
  constexpr bool kCanSplit = (P > 7);
  const bool split = kCanSplit && opt == SDG_OPT_OPT1;
  switch (what) {
    case 0: {
      const TendArgs& a = *static_cast<const TendArgs*>(args);
      return split ? launch_dqdt_impl<P, kCanSplit>(a, st) : launch_dqdt_impl<P, false>(a, st);
    }
    case 1: {
      const DivArgs& a = *static_cast<const DivArgs*>(args);
      return split ? launch_divlike_impl<P, kCanSplit>(a, st)
                   : launch_divlike_impl<P, false>(a, st);
    }
    case 3:
      return launch_gradlike_impl<P>(*static_cast<const DivArgs*>(args), st);
    default: {
      const DivArgs& a = *static_cast<const DivArgs*>(args);
      // lift: ox = out, D = Lift, ix = in
      return launch_lift_impl<P>(a.ox, a.D, a.ix, a.nelem, st);
    }
  }
}

}  // namespace sdg
