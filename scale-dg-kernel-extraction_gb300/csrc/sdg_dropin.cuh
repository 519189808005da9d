// Kernels behind the reference-shaped entry points, for meshes given as the
// reference's arrays (VMapM/VMapP with a halo buffer, normal_fn, Escale,
// Fscale), so any connectivity the caller builds is honoured.
//
//   flux_kernel      cal_elembnd_flux (mod_advect3d_eq.f90:89-142), one
//                    thread per face node, VMap indices range-checked;
//   dqdt_kernel      cal_dqdt (mod_advect3d_eq.f90:146-201), EPB elements
//                    per block staged in shared memory;
//   dqdt_eo_kernel   the same tendency with the even-odd line sums of the
//                    fused stage (opt type SDG_OPT_EVENODD), honouring the
//                    caller's per-node Escale and face fluxes;
//   divlike_kernel   tensorprod_divlike_dirXYZ (mod_dg_optr_kernel.f90:62-136)
//                    over a batch of elements;
//   lift_kernel      tensorprod_Lift_hexahedral (mod_dg_optr_kernel.f90:139-190).
#pragma once

#include "sdg_stage.cuh"
#include "sdg_stage_eo.cuh"

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

// Elements per block: as many whole elements as the block has threads for
// (32 at p = 1, 9 at p = 2, 4 at p = 3, 2 at p = 4, one from p = 5), so that
// every thread owns a node at low orders; R nodes a thread in all.
template <int P>
struct DropCfg {
  static constexpr int THREADS = (P >= 10) ? 512 : 256;
  static constexpr int EPB = (THREADS / Ord<P>::NP) > 0 ? THREADS / Ord<P>::NP : 1;
  static constexpr int R = (EPB * Ord<P>::NP + THREADS - 1) / THREADS;
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
  // one direction at a time, each node's running sum
  // Escale_x D F_x + Escale_y D F_y + Escale_z D F_z kept in acc: a thread
  // keeps one line sum live, not three (94 registers and two blocks an SM at
  // p = 3 with the three interleaved)
  constexpr int R = DropCfg<P>::R;
  double acc[R];
#pragma unroll
  for (int r = 0; r < R; r++) {
    const int t = threadIdx.x + r * T;
    if (t < nloc * NP) {
      const int le = t / NP, n = t - le * NP;
      const int j = (n / NQ) % NQ, k = n / NQ2;
      const double dx =
          line_sum<NQ, SPLIT3, NQ>(sD + n % NQ, fx + le * NP + j * NQ + k * NQ2, 1);
      acc[r] = a.Escale[g0 + t] * dx;
    }
  }
#pragma unroll
  for (int r = 0; r < R; r++) {
    const int t = threadIdx.x + r * T;
    if (t < nloc * NP) {
      const int le = t / NP, n = t - le * NP;
      const int i = n % NQ, j = (n / NQ) % NQ, k = n / NQ2;
      const double dy = line_sum<NQ, SPLIT3, 1>(sDt + j * NQ, fy + le * NP + i + k * NQ2, NQ);
      acc[r] = fma(a.Escale[g0 + t + NpNe], dy, acc[r]);
    }
  }
#pragma unroll
  for (int r = 0; r < R; r++) {
    const int t = threadIdx.x + r * T;
    if (t < nloc * NP) {
      const int le = t / NP, n = t - le * NP;
      const int i = n % NQ, j = (n / NQ) % NQ, k = n / NQ2;
      const double dz = line_sum<NQ, SPLIT3, 1>(sDt + k * NQ, fz + le * NP + i + j * NQ, NQ2);
      const double lf = lift_node<P>(a.Lift + n, a.flux + (eb + le) * NFT, i, j, k);
      a.dqdt[g0 + t] = -(fma(a.Escale[g0 + t + 2 * NpNe], dz, acc[r]) + lf);
    }
  }
}

// ---- even-odd cal_dqdt --------------------------------------------------

template <int P>
struct DqdtEoCfg {
  static constexpr int THREADS = 256;
  static constexpr int EPB = (256 / Ord<P>::NQ2) > 0 ? 256 / Ord<P>::NQ2 : 1;
};

template <int P>
constexpr size_t dqdt_eo_smem_bytes() {
  return sizeof(double) * (size_t)(3 * EoShape<P>::TE + DqdtEoCfg<P>::EPB * Ord<P>::NP) +
         2 * sizeof(unsigned long long);
}

// One line in pair form: s / d hold S(l) / Δ(l) (l < N/2), fm F(mid) for an
// odd N; T the direction's unscaled tables; gm / gp the caller's face fluxes
// of the line's - and + faces.  emit(m, dpart, lpart) receives, for position
// m, the derivative sum (times Escale by the caller) and the lift sum apart.
template <int P, typename Emit>
__device__ __forceinline__ void eo_line_dl(const double* row, const double* __restrict__ T,
                                           double gm, double gp, Emit&& emit) {
  using Sh = EoShape<P>;
  constexpr int N = Sh::N, H = Sh::H;
  double s[H], d[H];
#pragma unroll
  for (int l = 0; l < H; l++) {
    s[l] = row[l];
    d[l] = row[N - 1 - l];
  }
  double fm = 0.0;
  if constexpr (Sh::ODD != 0) fm = row[H];
  const double gs = gm + gp, gd = gm - gp;
  constexpr int kRowUnroll = (N <= 5) ? H : 1;
#pragma unroll kRowUnroll
  for (int i = 0; i < H; i++) {
    double e = T[Sh::OFF_E + i * H] * s[0];
#pragma unroll
    for (int l = 1; l < H; l++) e = fma(T[Sh::OFF_E + i * H + l], s[l], e);
    if constexpr (Sh::ODD != 0) e = fma(T[Sh::OFF_DM + i], fm, e);
    double o = T[Sh::OFF_O + i * H] * d[0];
#pragma unroll
    for (int l = 1; l < H; l++) o = fma(T[Sh::OFF_O + i * H + l], d[l], o);
    const double le = T[Sh::OFF_B + i] * gd, lo = T[Sh::OFF_A + i] * gs;
    emit(i, e + o, lo + le);
    emit(N - 1 - i, o - e, lo - le);
  }
  if constexpr (Sh::ODD != 0) {
    double o = T[Sh::OFF_O + H * H] * d[0];
#pragma unroll
    for (int l = 1; l < H; l++) o = fma(T[Sh::OFF_O + H * H + l], d[l], o);
    emit(H, o, T[Sh::OFF_A + H] * gs);
  }
}

// cal_dqdt (mod_advect3d_eq.f90:146-201) with the even-odd factorisation:
// per line the divergence sum D F is formed from the pair values and the two
// faces' lift from the lift columns, dqdt = -(sum_d (Escale_d * D_d F_d +
// lift_d)).  Every block builds the unscaled tables from D1D and Lift_mat
// (the lift column of a face from its tangential node (0, 0)); block 0 checks
// the symmetries the factorisation needs -- D1D centro-antisymmetric, D1D_tr
// its transpose, each face's lift constant over the tangential nodes, the +
// face's column the mirror of the - face's, all to 1e-13 of the largest entry
// -- and sets *err = 2 when one fails.  The summation order is neither
// GENERAL's nor OPT1's; results agree with both to rounding.
template <int P>
__global__ void __launch_bounds__(DqdtEoCfg<P>::THREADS, 4) dqdt_eo_kernel(const TendArgs a) {
  using O = Ord<P>;
  using Sh = EoShape<P>;
  constexpr int NQ = O::NQ, NQ2 = O::NQ2, NP = O::NP, NFP = O::NFP, NFT = O::NFT,
                EPB = DqdtEoCfg<P>::EPB, T = DqdtEoCfg<P>::THREADS, TE = Sh::TE, N = Sh::N,
                H = Sh::H, HR = Sh::HR;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* sT = reinterpret_cast<double*>(smem_raw);  // [3][TE]
  double* sA = sT + 3 * TE;                          // [EPB][NP]: x pairs, then sums
  unsigned long long* smax = reinterpret_cast<unsigned long long*>(sA + EPB * NP);
  const long long eb = (long long)blockIdx.x * EPB;
  const int nloc = (int)min((long long)EPB, (long long)a.Ne - eb);
  if (nloc <= 0) return;
  const double* __restrict__ D = a.D;
  const double* __restrict__ L = a.Lift;
  auto Dv = [&](int i, int l) { return D[i + l * N]; };  // D1D(i,l), column-major
  auto Ds = [&](int i, int l) { return 0.5 * (Dv(i, l) - Dv(N - 1 - i, N - 1 - l)); };
  // lift of face f at normal index m (tangential indices 0, 0) on axis ax
  auto node = [](int ax, int m, int t1, int t2) {
    return (ax == 0) ? m + NQ * t1 + NQ2 * t2 : (ax == 1) ? t1 + NQ * m + NQ2 * t2
                                                           : t1 + NQ * t2 + NQ2 * m;
  };
  auto col = [&](int ax, int side, int m) {
    const int f = (ax == 0) ? (side ? 1 : 3) : (ax == 1) ? (side ? 2 : 0) : (side ? 5 : 4);
    return L[node(ax, m, 0, 0) + (long long)f * NP];
  };
  auto lam = [&](int ax, int m) { return 0.5 * (col(ax, 0, m) + col(ax, 1, N - 1 - m)); };
  for (int t = threadIdx.x; t < 3 * TE; t += T) {
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
    sT[t] = v;
  }
  if (blockIdx.x == 0) {
    // the largest |D| and |Lift| (non-negative doubles order like their bits)
    if (threadIdx.x == 0) smax[0] = smax[1] = 0ull;
    __syncthreads();
    unsigned long long mD = 0, mL = 0;
    for (int t = threadIdx.x; t < NQ2; t += T) mD = max(mD, (unsigned long long)__double_as_longlong(fabs(D[t])));
    for (int t = threadIdx.x; t < 6 * NP; t += T) mL = max(mL, (unsigned long long)__double_as_longlong(fabs(L[t])));
    atomicMax(&smax[0], mD);
    atomicMax(&smax[1], mL);
    __syncthreads();
    const double tD = 1e-13 * __longlong_as_double((long long)smax[0]);
    const double tL = 1e-13 * __longlong_as_double((long long)smax[1]);
    bool bad = false;
    for (int t = threadIdx.x; t < NQ2; t += T) {
      const int i = t % N, l = t / N;
      bad |= fabs(Dv(i, l) + Dv(N - 1 - i, N - 1 - l)) > tD;
      bad |= fabs(a.Dt[l + i * N] - Dv(i, l)) > tD;
    }
    for (int t = threadIdx.x; t < 6 * NP; t += T) {
      const int f = t / NP, n = t - f * NP;
      const int ax = (f == 1 || f == 3) ? 0 : (f == 0 || f == 2) ? 1 : 2;
      const int side = (f == 1 || f == 2 || f == 5) ? 1 : 0;
      const int c[3] = {n % NQ, (n / NQ) % NQ, n / NQ2};
      bad |= fabs(L[t] - col(ax, side, c[ax])) > tL;
      if (n < N && ax == 0 && side == 0)  // mirror, once per axis below
        for (int x = 0; x < 3; x++) bad |= fabs(col(x, 0, n) - col(x, 1, N - 1 - n)) > tL;
    }
    if (bad) atomicExch(a.err, 2);
  }
  const long long g0 = eb * NP;
  const double* __restrict__ q = a.q;
  // x pair values: one task per (element, x line, c < ceil(N/2))
  for (int t = threadIdx.x; t < nloc * NQ2 * HR; t += T) {
    const int le = t / (NQ2 * HR), w = t - le * NQ2 * HR;
    const int r = w / HR, c = w - r * HR;
    const long long g = g0 + (long long)le * NP + (long long)r * NQ;
    double* row = sA + le * NP + r * NQ;
    if (c < H) {
      const double q1 = q[g + c], u1 = a.u[g + c];
      const double p2 = q[g + NQ - 1 - c] * a.u[g + NQ - 1 - c];
      row[c] = fma(q1, u1, p2);
      row[NQ - 1 - c] = fma(q1, u1, -p2);
    } else {
      row[c] = q[g + c] * a.u[g + c];
    }
  }
  __syncthreads();
  const long long NpNe = (long long)NP * a.Ne;
  const int r = threadIdx.x % NQ2, le = threadIdx.x / NQ2;
  const bool has_line = threadIdx.x < nloc * NQ2;
  const double* fl = a.flux + (eb + le) * NFT + r;
  // x lines: faces -x (3) and +x (1); results over the pair values
  if (has_line) {
    double* row = sA + le * NP + r * NQ;
    const long long g = g0 + (long long)le * NP + (long long)r * NQ;
    eo_line_dl<P>(row, sT, fl[3 * NFP], fl[1 * NFP], [&](int m, double vd, double vl) {
      row[m] = fma(a.Escale[g + m], vd, vl);
    });
  }
  __syncthreads();
  // y lines: faces -y (0) and +y (2); added into the sums
  if (has_line) {
    const int off = le * NP + (r % NQ) + (r / NQ) * NQ2;
    double row[NQ];
    eo_pairs_f64<P>(q, a.v, g0 + off, NQ, row);
    eo_line_dl<P>(row, sT + TE, fl[0], fl[2 * NFP], [&](int m, double vd, double vl) {
      const int n = off + m * NQ;
      sA[n] += fma(a.Escale[g0 + n + NpNe], vd, vl);
    });
  }
  __syncthreads();
  // z lines: faces -z (4) and +z (5); finish the node
  if (has_line) {
    const int off = le * NP + r;
    double row[NQ];
    eo_pairs_f64<P>(q, a.w, g0 + off, NQ2, row);
    eo_line_dl<P>(row, sT + 2 * TE, fl[4 * NFP], fl[5 * NFP], [&](int m, double vd, double vl) {
      const int n = off + m * NQ2;
      a.dqdt[g0 + n] = -(sA[n] + fma(a.Escale[g0 + n + 2 * NpNe], vd, vl));
    });
  }
}

template <int P>
int launch_dqdt_eo_impl(const TendArgs& a, cudaStream_t st) {
  constexpr size_t smem = dqdt_eo_smem_bytes<P>();
  SDG_CUDA_TRY(cudaFuncSetAttribute(dqdt_eo_kernel<P>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const long long nblk = ((long long)a.Ne + DqdtEoCfg<P>::EPB - 1) / DqdtEoCfg<P>::EPB;
  if (nblk == 0) return SDG_OK;
  dqdt_eo_kernel<P><<<(unsigned)nblk, DqdtEoCfg<P>::THREADS, smem, st>>>(a);
  SDG_CUDA_TRY(cudaGetLastError());
  return SDG_OK;
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
  // one direction at a time (a thread keeps one line sum live; 74 registers
  // at p = 3 with the three interleaved)
  for (int t = threadIdx.x; t < nloc * NP; t += T) {
    const int le = t / NP, n = t - le * NP;
    const int j = (n / NQ) % NQ, k = n / NQ2;
    a.ox[g0 + t] = line_sum<NQ, SPLIT3, NQ>(sD + n % NQ, fx + le * NP + j * NQ + k * NQ2, 1);
  }
  for (int t = threadIdx.x; t < nloc * NP; t += T) {
    const int le = t / NP, n = t - le * NP;
    const int i = n % NQ, j = (n / NQ) % NQ, k = n / NQ2;
    a.oy[g0 + t] = line_sum<NQ, SPLIT3, 1>(sDt + j * NQ, fy + le * NP + i + k * NQ2, NQ);
  }
  for (int t = threadIdx.x; t < nloc * NP; t += T) {
    const int le = t / NP, n = t - le * NP;
    const int i = n % NQ, j = (n / NQ) % NQ;
    a.oz[g0 + t] = line_sum<NQ, SPLIT3, 1>(sDt + (n / NQ2) * NQ, fz + le * NP + i + j * NQ, NQ2);
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
  // one direction at a time: a thread keeps one running sum live, not three
  // (82 registers and three blocks an SM at p = 7 when the three were
  // interleaved)
  if (a.ox)
    for (int t = threadIdx.x; t < nloc * NP; t += T) {
      const int le = t / NP, n = t - le * NP;
      const int i = n % NQ, j = (n / NQ) % NQ, k = n / NQ2;
      a.ox[g0 + t] = line_sum<NQ, false, NQ>(sD + i, f + le * NP + j * NQ + k * NQ2, 1);
    }
  if (a.oy)
    for (int t = threadIdx.x; t < nloc * NP; t += T) {
      const int le = t / NP, n = t - le * NP;
      const int i = n % NQ, j = (n / NQ) % NQ, k = n / NQ2;
      a.oy[g0 + t] = line_sum<NQ, false, 1>(sDt + j * NQ, f + le * NP + i + k * NQ2, NQ);
    }
  if (a.oz)
    for (int t = threadIdx.x; t < nloc * NP; t += T) {
      const int le = t / NP, n = t - le * NP;
      const int i = n % NQ, j = (n / NQ) % NQ, k = n / NQ2;
      a.oz[g0 + t] = line_sum<NQ, false, 1>(sDt + k * NQ, f + le * NP + i + j * NQ, NQ2);
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

}  // namespace sdg

#include "sdg_dropin_step.cuh"

namespace sdg {

// Tables of the fused reference-array stage (one block, symmetry checks).
struct StepTablesArgs {
  const double* D;
  const double* Dt;
  const double* Lift;
  double* tab;
  int* err;
};

// Per-order entry used by the dispatch in sdg_dropin.cu.  what: 0 cal_dqdt,
// 1 divlike, 2 lift, 3 gradlike, 4 one fused reference-array stage, 5 the
// tables of that stage.
template <int P>
int dropin_order(int what, int opt, const void* args, cudaStream_t st) {
  constexpr bool kCanSplit = (P > 7);
  const bool split = kCanSplit && opt == SDG_OPT_OPT1;
  switch (what) {
    case 0: {
      const TendArgs& a = *static_cast<const TendArgs*>(args);
      if (opt == SDG_OPT_EVENODD) return launch_dqdt_eo_impl<P>(a, st);
      return split ? launch_dqdt_impl<P, kCanSplit>(a, st) : launch_dqdt_impl<P, false>(a, st);
    }
    case 1: {
      const DivArgs& a = *static_cast<const DivArgs*>(args);
      return split ? launch_divlike_impl<P, kCanSplit>(a, st)
                   : launch_divlike_impl<P, false>(a, st);
    }
    case 3:
      return launch_gradlike_impl<P>(*static_cast<const DivArgs*>(args), st);
    case 4:
      return launch_step_ref_impl<P>(*static_cast<const StepRefArgs*>(args), st);
    case 5: {
      const StepTablesArgs& a = *static_cast<const StepTablesArgs*>(args);
      step_tables_kernel<P><<<1, 256, 0, st>>>(a.D, a.Dt, a.Lift, a.tab, a.err);
      SDG_CUDA_TRY(cudaGetLastError());
      return SDG_OK;
    }
    default: {
      const DivArgs& a = *static_cast<const DivArgs*>(args);
      // lift: ox = out, D = Lift, ix = in
      return launch_lift_impl<P>(a.ox, a.D, a.ix, a.nelem, st);
    }
  }
}

}  // namespace sdg
