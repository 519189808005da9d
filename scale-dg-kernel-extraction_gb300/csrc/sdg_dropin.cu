// Reference-shaped entry points: advect3d_eq_cal_tend, the two DG operators,
// update_halo and the RK combine, on host or device pointers.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <vector>

#include "sdg_dropin.cuh"

namespace sdg {

#define SDG_DECL_DROPIN(p) \
  int dropin_p##p(int what, int opt, const void* args, cudaStream_t st);
SDG_DECL_DROPIN(1) SDG_DECL_DROPIN(2) SDG_DECL_DROPIN(3) SDG_DECL_DROPIN(4)
SDG_DECL_DROPIN(5) SDG_DECL_DROPIN(6) SDG_DECL_DROPIN(7) SDG_DECL_DROPIN(8)
SDG_DECL_DROPIN(9) SDG_DECL_DROPIN(10) SDG_DECL_DROPIN(11) SDG_DECL_DROPIN(12)
SDG_DECL_DROPIN(13) SDG_DECL_DROPIN(14) SDG_DECL_DROPIN(15)
#undef SDG_DECL_DROPIN

// what: 0 = cal_dqdt, 1 = divlike, 2 = lift, 3 = gradlike (mod_dg_optr_kernel.f90:87-133
// and :155-186 select the per-order kernel the same way).
static int dropin(int p, int what, int opt, const void* args, cudaStream_t st) {
  switch (p) {
    case 1: return dropin_p1(what, opt, args, st);
    case 2: return dropin_p2(what, opt, args, st);
    case 3: return dropin_p3(what, opt, args, st);
    case 4: return dropin_p4(what, opt, args, st);
    case 5: return dropin_p5(what, opt, args, st);
    case 6: return dropin_p6(what, opt, args, st);
    case 7: return dropin_p7(what, opt, args, st);
    case 8: return dropin_p8(what, opt, args, st);
    case 9: return dropin_p9(what, opt, args, st);
    case 10: return dropin_p10(what, opt, args, st);
    case 11: return dropin_p11(what, opt, args, st);
    case 12: return dropin_p12(what, opt, args, st);
    case 13: return dropin_p13(what, opt, args, st);
    case 14: return dropin_p14(what, opt, args, st);
    case 15: return dropin_p15(what, opt, args, st);
    default: return fail(SDG_ERR_UNSUPPORTED_ORDER, "PolyOrder %d outside 1..15", p);
  }
}

// GENERAL and OPT1 as the reference; EVENODD selects the even-odd tendency
// kernel in cal_tend and the GENERAL order in the operator entry points.
static int check_opt(int opt) {
  if (opt != SDG_OPT_GENERAL && opt != SDG_OPT_OPT1 && opt != SDG_OPT_EVENODD)
    return fail(SDG_ERR_BAD_OPTTYPE,
                "DGOptrKernel type not set (call sdg_dg_optr_kernel_setup) or "
                "unknown (%d)", opt);
  return SDG_OK;
}

static int check_order(int Nq) {
  if (Nq - 1 < 1 || Nq - 1 > kMaxOrder)
    return fail(SDG_ERR_UNSUPPORTED_ORDER, "PolyOrder %d outside 1..15", Nq - 1);
  return SDG_OK;
}

static int check_tend_shape(int Nq, int Np, int NfpTot, int Ne, int NeA) {
  SDG_TRY(check_order(Nq));
  if (Np != Nq * Nq * Nq || NfpTot != 6 * Nq * Nq || Ne < 0 || NeA < Ne)
    return fail(SDG_ERR_INVALID_ARG,
                "inconsistent sizes Nq=%d Np=%d NfpTot=%d Ne=%d NeA=%d", Nq, Np,
                NfpTot, Ne, NeA);
  return SDG_OK;
}

// One device allocation carved into aligned pieces; freed on scope exit.
class Arena {
 public:
  ~Arena() {
    if (base_) cudaFree(base_);
  }
  size_t add(size_t bytes) {
    const size_t off = size_;
    size_ += (bytes + 255) & ~size_t(255);
    return off;
  }
  int alloc() {
    if (size_ == 0) return SDG_OK;
    SDG_CUDA_TRY(cudaMalloc(&base_, size_));
    return SDG_OK;
  }
  template <typename T>
  T* at(size_t off) const { return reinterpret_cast<T*>(static_cast<char*>(base_) + off); }

 private:
  void* base_ = nullptr;
  size_t size_ = 0;
};

// cal_elembnd_flux, mod_advect3d_eq.f90:116-140, one thread per face node.
__global__ void flux_kernel(const TendArgs a, int NfpTot) {
  const long long NT = (long long)NfpTot * a.Ne;
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < NT;
       m += (long long)gridDim.x * blockDim.x) {
    const long long iM = (long long)a.VMapM[m] - 1, iP = (long long)a.VMapP[m] - 1;
    if (iM < 0 || iM >= a.NpNeA || iP < 0 || iP >= a.NpNeA) {
      atomicExch(a.err, 1);
      a.flux[m] = 0.0;
      continue;
    }
    const double n1 = a.normal_fn[m], n2 = a.normal_fn[m + NT],
                 n3 = a.normal_fn[m + 2 * NT];
    const double qM = a.q[iM], qP = a.q[iP];
    // all six velocity gathers are independent of the normals, so they are
    // in flight together (a branch on the normal's axis that gathered one
    // component per side measured 3 % slower: its gathers waited on the
    // normal loads)
    const double VelM = a.u[iM] * n1 + a.v[iM] * n2 + a.w[iM] * n3;
    const double VelP = a.u[iP] * n1 + a.v[iP] * n2 + a.w[iP] * n3;
    const double alpha = 0.5 * fabs(VelP + VelM);
    a.flux[m] = (0.5 * a.Fscale[m]) * ((qP * VelP - qM * VelM) - alpha * (qP - qM));
  }
}

int tend_dev(const TendArgs& a, int p, int NfpTot, int opt, cudaStream_t st) {
  if (a.Ne == 0) return SDG_OK;
  const long long NT = (long long)NfpTot * a.Ne;
  long long nb = (NT + 255) / 256;
  if (nb > 152LL * 64) nb = 152LL * 64;
  flux_kernel<<<(unsigned)nb, 256, 0, st>>>(a, NfpTot);
  SDG_CUDA_TRY(cudaGetLastError());
  return dropin(p, 0, opt, &a, st);
}

}  // namespace sdg

using namespace sdg;

namespace {

__global__ void update_halo_kernel(double* f, const int* map, long long base,
                                   long long nhalo, long long limit, int* err) {
  for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < nhalo;
       b += (long long)gridDim.x * blockDim.x) {
    const long long src = (long long)map[b] - 1;
    if (src < 0 || src >= limit) {
      if (err) atomicExch(err, 1);
      continue;
    }
    f[base + b] = f[src];
  }
}

__global__ void rk_kernel(double* q, const double* q0, const double* dqdt,
                          long long n, double a, double b, double dt) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    // main.f90:70-71: rk_a*q0 + rk_b*(q + dt*dqdt)
    const double r = b * (q[i] + dt * dqdt[i]);
    q[i] = (a != 0.0) ? a * q0[i] + r : r;
  }
}

// Once per call, one thread per face node m: the owned nodes its qM and qP
// come from (VMapM(m), VMapP(m), a halo slot b followed through
// halo_src_map(b)) and the velocity factors (tP, tM) of its flux from the
// caller's velocity at VMapM / VMapP, normal_fn and Fscale.  An entry out of
// range sets *err = 1 and gives the face node a zero flux.
__global__ void step_face_kernel(const int* __restrict__ VMapM, const int* __restrict__ VMapP,
                                 const int* __restrict__ halo_src_map,
                                 const double* __restrict__ u, const double* __restrict__ v,
                                 const double* __restrict__ w,
                                 const double* __restrict__ normal_fn,
                                 const double* __restrict__ Fscale, int2* res, double2* fc,
                                 long long NT, long long NpNe, long long NpNeA,
                                 long long NhaloNode, int* err) {
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < NT;
       m += (long long)gridDim.x * blockDim.x) {
    const long long vM = (long long)VMapM[m] - 1, vP = (long long)VMapP[m] - 1;
    long long r[2] = {vM, vP};
#pragma unroll
    for (int side = 0; side < 2; side++)
      if (r[side] >= NpNe && r[side] < NpNeA && r[side] - NpNe < NhaloNode)
        r[side] = (long long)halo_src_map[r[side] - NpNe] - 1;
    const bool ok = vM >= 0 && vM < NpNeA && vP >= 0 && vP < NpNeA && r[0] >= 0 &&
                    r[0] < NpNe && r[1] >= 0 && r[1] < NpNe;
    if (!ok) {
      atomicExch(err, 1);
      res[m] = make_int2(-1, -1);
      fc[m] = make_double2(0.0, 0.0);
      continue;
    }
    res[m] = make_int2((int)r[0], (int)r[1]);
    const double n1 = normal_fn[m], n2 = normal_fn[m + NT], n3 = normal_fn[m + 2 * NT];
    const double velM = u[vM] * n1 + v[vM] * n2 + w[vM] * n3;
    const double velP = u[vP] * n1 + v[vP] * n2 + w[vP] * n3;
    const double alpha = 0.5 * fabs(velP + velM);
    const double hf = 0.5 * Fscale[m];
    fc[m] = make_double2(hf * (velP - alpha), hf * (velM - alpha));
  }
}

// Once per call, one warp per element: whether the element's Escale is one
// value per direction over all its nodes (compared bit for bit), stored as
// (Es_x, Es_y, Es_z, 1), else (.., 0).
__global__ void step_escale_kernel(const double* __restrict__ Es, double4* esu, long long Ne,
                                   int Np) {
  const long long NpNe = (long long)Np * Ne;
  const int lane = threadIdx.x & 31;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long e = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; e < Ne;
       e += nwarps) {
    double v[3];
    bool same = true;
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const double* x = Es + e * Np + d * NpNe;
      v[d] = x[0];
      const long long b = __double_as_longlong(v[d]);
      for (int n = lane; n < Np; n += 32) same &= (__double_as_longlong(x[n]) == b);
    }
    same = __all_sync(0xffffffffu, same);
    if (lane == 0) esu[e] = make_double4(v[0], v[1], v[2], same ? 1.0 : 0.0);
  }
}

unsigned grid_for(long long n) {
  long long nb = (n + 255) / 256;
  if (nb > 152LL * 64) nb = 152LL * 64;
  return (unsigned)(nb > 0 ? nb : 1);
}

}  // namespace

extern "C" {

int sdg_advect3d_eq_cal_tend_dev(double* dqdt, const double* q, const double* u,
                                 const double* v, const double* w,
                                 const double* D1D, const double* D1D_tr,
                                 const double* Lift_mat, const int* VMapM,
                                 const int* VMapP, const double* normal_fn,
                                 const double* Escale, const double* Fscale,
                                 int Nq, int Np, int NfpTot, int Ne, int NeA,
                                 int opt, double* flux_scratch, int* err_flag,
                                 void* stream) {
  SDG_TRY(check_opt(opt));
  SDG_TRY(check_tend_shape(Nq, Np, NfpTot, Ne, NeA));
  if (Ne == 0) return SDG_OK;
  if (!dqdt || !q || !u || !v || !w || !D1D || !D1D_tr || !Lift_mat || !VMapM ||
      !VMapP || !normal_fn || !Escale || !Fscale || !flux_scratch || !err_flag)
    return fail(SDG_ERR_INVALID_ARG, "NULL device pointer");
  TendArgs a{dqdt, q, u, v, w, D1D, D1D_tr, Lift_mat, VMapM, VMapP, normal_fn,
             Escale, Fscale, flux_scratch, err_flag, Ne, (long long)Np * NeA};
  return tend_dev(a, Nq - 1, NfpTot, opt, as_stream(stream));
}

int sdg_advect3d_eq_cal_tend(double* dqdt, const double* q, const double* u,
                             const double* v, const double* w, const double* D1D,
                             const double* D1D_tr, const double* Lift_mat,
                             const int* VMapM, const int* VMapP,
                             const double* normal_fn, const double* Escale,
                             const double* Fscale, int Nq, int Np, int NfpTot,
                             int Ne, int NeA) {
  const int opt = sdg_dg_optr_kernel_type();
  SDG_TRY(check_opt(opt));
  SDG_TRY(check_tend_shape(Nq, Np, NfpTot, Ne, NeA));
  if (Ne == 0) return SDG_OK;
  if (!dqdt || !q || !u || !v || !w || !D1D || !D1D_tr || !Lift_mat || !VMapM ||
      !VMapP || !normal_fn || !Escale || !Fscale)
    return fail(SDG_ERR_INVALID_ARG, "NULL host pointer");
  SDG_TRY(require_device());
  const size_t nA = (size_t)Np * NeA, nO = (size_t)Np * Ne, nF = (size_t)NfpTot * Ne,
               nD = (size_t)Nq * Nq, nL = 6 * (size_t)Np;
  Arena ar;
  const size_t oq = ar.add(8 * nA), ou = ar.add(8 * nA), ov = ar.add(8 * nA),
               ow = ar.add(8 * nA), od = ar.add(8 * nO), oD = ar.add(8 * nD),
               oDt = ar.add(8 * nD), oL = ar.add(8 * nL), oM = ar.add(4 * nF),
               oP = ar.add(4 * nF), oN = ar.add(8 * 3 * nF), oE = ar.add(8 * 3 * nO),
               oS = ar.add(8 * nF), oX = ar.add(8 * nF), oR = ar.add(sizeof(int));
  SDG_TRY(ar.alloc());
  cudaStream_t st = nullptr;
  SDG_CUDA_TRY(cudaMemcpyAsync(ar.at<void>(oq), q, 8 * nA, cudaMemcpyHostToDevice, st));
  SDG_CUDA_TRY(cudaMemcpyAsync(ar.at<void>(ou), u, 8 * nA, cudaMemcpyHostToDevice, st));
  SDG_CUDA_TRY(cudaMemcpyAsync(ar.at<void>(ov), v, 8 * nA, cudaMemcpyHostToDevice, st));
  SDG_CUDA_TRY(cudaMemcpyAsync(ar.at<void>(ow), w, 8 * nA, cudaMemcpyHostToDevice, st));
  SDG_CUDA_TRY(cudaMemcpyAsync(ar.at<void>(oD), D1D, 8 * nD, cudaMemcpyHostToDevice, st));
  SDG_CUDA_TRY(cudaMemcpyAsync(ar.at<void>(oDt), D1D_tr, 8 * nD, cudaMemcpyHostToDevice, st));
  SDG_CUDA_TRY(cudaMemcpyAsync(ar.at<void>(oL), Lift_mat, 8 * nL, cudaMemcpyHostToDevice, st));
  SDG_CUDA_TRY(cudaMemcpyAsync(ar.at<void>(oM), VMapM, 4 * nF, cudaMemcpyHostToDevice, st));
  SDG_CUDA_TRY(cudaMemcpyAsync(ar.at<void>(oP), VMapP, 4 * nF, cudaMemcpyHostToDevice, st));
  SDG_CUDA_TRY(cudaMemcpyAsync(ar.at<void>(oN), normal_fn, 8 * 3 * nF, cudaMemcpyHostToDevice, st));
  SDG_CUDA_TRY(cudaMemcpyAsync(ar.at<void>(oE), Escale, 8 * 3 * nO, cudaMemcpyHostToDevice, st));
  SDG_CUDA_TRY(cudaMemcpyAsync(ar.at<void>(oS), Fscale, 8 * nF, cudaMemcpyHostToDevice, st));
  SDG_CUDA_TRY(cudaMemsetAsync(ar.at<void>(oR), 0, sizeof(int), st));
  TendArgs a{ar.at<double>(od), ar.at<double>(oq), ar.at<double>(ou),
             ar.at<double>(ov), ar.at<double>(ow), ar.at<double>(oD),
             ar.at<double>(oDt), ar.at<double>(oL), ar.at<int>(oM),
             ar.at<int>(oP), ar.at<double>(oN), ar.at<double>(oE),
             ar.at<double>(oS), ar.at<double>(oX), ar.at<int>(oR), Ne,
             (long long)Np * NeA};
  SDG_TRY(tend_dev(a, Nq - 1, NfpTot, opt, st));
  int err = 0;
  SDG_CUDA_TRY(cudaMemcpyAsync(&err, ar.at<void>(oR), sizeof(int), cudaMemcpyDeviceToHost, st));
  SDG_CUDA_TRY(cudaMemcpyAsync(dqdt, ar.at<void>(od), 8 * nO, cudaMemcpyDeviceToHost, st));
  SDG_CUDA_TRY(cudaStreamSynchronize(st));
  if (err == 2)
    return fail(SDG_ERR_INVALID_ARG,
                "D1D / D1D_tr / Lift_mat lack the even-odd symmetries; use GENERAL or OPT1");
  if (err) return fail(SDG_ERR_MESH, "a VMapM/VMapP entry is outside 1..Np*NeA");
  return SDG_OK;
}

int sdg_tensorprod_divlike_dirXYZ_dev(double* ox, double* oy, double* oz,
                                      const double* Mat, const double* Mat_tr,
                                      const double* ix, const double* iy,
                                      const double* iz, int Nq, int nelem,
                                      int opt, void* stream) {
  SDG_TRY(check_opt(opt));
  SDG_TRY(check_order(Nq));
  if (nelem < 0) return fail(SDG_ERR_INVALID_ARG, "nelem < 0");
  if (nelem == 0) return SDG_OK;
  if (!ox || !oy || !oz || !Mat || !Mat_tr || !ix || !iy || !iz)
    return fail(SDG_ERR_INVALID_ARG, "NULL device pointer");
  DivArgs a{ox, oy, oz, Mat, Mat_tr, ix, iy, iz, nelem};
  return dropin(Nq - 1, 1, opt, &a, as_stream(stream));
}

int sdg_tensorprod_divlike_dirXYZ(double* ox, double* oy, double* oz,
                                  const double* Mat, const double* Mat_tr,
                                  const double* ix, const double* iy,
                                  const double* iz, int Nq, int nelem) {
  const int opt = sdg_dg_optr_kernel_type();
  SDG_TRY(check_opt(opt));
  SDG_TRY(check_order(Nq));
  if (nelem < 0) return fail(SDG_ERR_INVALID_ARG, "nelem < 0");
  if (nelem == 0) return SDG_OK;
  if (!ox || !oy || !oz || !Mat || !Mat_tr || !ix || !iy || !iz)
    return fail(SDG_ERR_INVALID_ARG, "NULL host pointer");
  SDG_TRY(require_device());
  const size_t n = (size_t)Nq * Nq * Nq * nelem, nD = (size_t)Nq * Nq;
  Arena ar;
  const size_t o[8] = {ar.add(8 * n), ar.add(8 * n), ar.add(8 * n), ar.add(8 * nD),
                       ar.add(8 * nD), ar.add(8 * n), ar.add(8 * n), ar.add(8 * n)};
  SDG_TRY(ar.alloc());
  const double* hin[5] = {Mat, Mat_tr, ix, iy, iz};
  const size_t sz[5] = {nD, nD, n, n, n};
  for (int t = 0; t < 5; t++)
    SDG_CUDA_TRY(cudaMemcpy(ar.at<void>(o[3 + t]), hin[t], 8 * sz[t], cudaMemcpyHostToDevice));
  DivArgs a{ar.at<double>(o[0]), ar.at<double>(o[1]), ar.at<double>(o[2]),
            ar.at<double>(o[3]), ar.at<double>(o[4]), ar.at<double>(o[5]),
            ar.at<double>(o[6]), ar.at<double>(o[7]), nelem};
  SDG_TRY(dropin(Nq - 1, 1, opt, &a, nullptr));
  SDG_CUDA_TRY(cudaMemcpy(ox, a.ox, 8 * n, cudaMemcpyDeviceToHost));
  SDG_CUDA_TRY(cudaMemcpy(oy, a.oy, 8 * n, cudaMemcpyDeviceToHost));
  SDG_CUDA_TRY(cudaMemcpy(oz, a.oz, 8 * n, cudaMemcpyDeviceToHost));
  return SDG_OK;
}

// gradlike_dirXYZ (erb:166-219): one input field, three outputs.
int sdg_tensorprod_gradlike_dirXYZ_dev(double* ox, double* oy, double* oz, const double* Mat,
                                       const double* Mat_tr, const double* in, int Nq,
                                       int nelem, void* stream) {
  SDG_TRY(check_order(Nq));
  if (nelem < 0) return fail(SDG_ERR_INVALID_ARG, "nelem < 0");
  if (nelem == 0) return SDG_OK;
  if (!ox || !oy || !oz || !Mat || !Mat_tr || !in)
    return fail(SDG_ERR_INVALID_ARG, "NULL device pointer");
  DivArgs a{ox, oy, oz, Mat, Mat_tr, in, nullptr, nullptr, nelem};
  return dropin(Nq - 1, 3, SDG_OPT_GENERAL, &a, as_stream(stream));
}

// divlike_dirXYZ_var5 (erb:347-465): five variables per element, each the
// OPT1-order divlike contraction; the (Nq,Nq,Nq,5) element blocks make the
// call the divlike kernel over 5*nelem consecutive Nq^3 blocks.
int sdg_tensorprod_divlike_dirXYZ_var5_dev(double* ox, double* oy, double* oz,
                                           const double* Mat, const double* Mat_tr,
                                           const double* ix, const double* iy,
                                           const double* iz, int Nq, int nelem,
                                           void* stream) {
  SDG_TRY(check_order(Nq));
  if (nelem < 0 || nelem > 0x7fffffff / 5) return fail(SDG_ERR_INVALID_ARG, "bad nelem %d", nelem);
  if (nelem == 0) return SDG_OK;
  if (!ox || !oy || !oz || !Mat || !Mat_tr || !ix || !iy || !iz)
    return fail(SDG_ERR_INVALID_ARG, "NULL device pointer");
  DivArgs a{ox, oy, oz, Mat, Mat_tr, ix, iy, iz, 5 * nelem};
  return dropin(Nq - 1, 1, SDG_OPT_OPT1, &a, as_stream(stream));
}

namespace {
// Host-pointer wrapper shared by gradlike and var5: copies nin inputs of n
// doubles and the two Nq x Nq matrices in, runs `what`, copies 3 outputs out.
int host_contract(int what, double* ox, double* oy, double* oz, const double* Mat,
                  const double* Mat_tr, const double* const* in, int nin, int Nq, int nblocks,
                  int opt) {
  SDG_TRY(require_device());
  const size_t n = (size_t)Nq * Nq * Nq * nblocks, nD = (size_t)Nq * Nq;
  Arena ar;
  size_t o[8];
  for (int t = 0; t < 3; t++) o[t] = ar.add(8 * n);
  o[3] = ar.add(8 * nD);
  o[4] = ar.add(8 * nD);
  for (int t = 0; t < nin; t++) o[5 + t] = ar.add(8 * n);
  SDG_TRY(ar.alloc());
  SDG_CUDA_TRY(cudaMemcpy(ar.at<void>(o[3]), Mat, 8 * nD, cudaMemcpyHostToDevice));
  SDG_CUDA_TRY(cudaMemcpy(ar.at<void>(o[4]), Mat_tr, 8 * nD, cudaMemcpyHostToDevice));
  for (int t = 0; t < nin; t++)
    SDG_CUDA_TRY(cudaMemcpy(ar.at<void>(o[5 + t]), in[t], 8 * n, cudaMemcpyHostToDevice));
  DivArgs a{ar.at<double>(o[0]), ar.at<double>(o[1]), ar.at<double>(o[2]),
            ar.at<double>(o[3]), ar.at<double>(o[4]), ar.at<double>(o[5]),
            nin > 1 ? ar.at<double>(o[6]) : nullptr, nin > 2 ? ar.at<double>(o[7]) : nullptr,
            nblocks};
  SDG_TRY(dropin(Nq - 1, what, opt, &a, nullptr));
  SDG_CUDA_TRY(cudaMemcpy(ox, a.ox, 8 * n, cudaMemcpyDeviceToHost));
  SDG_CUDA_TRY(cudaMemcpy(oy, a.oy, 8 * n, cudaMemcpyDeviceToHost));
  SDG_CUDA_TRY(cudaMemcpy(oz, a.oz, 8 * n, cudaMemcpyDeviceToHost));
  return SDG_OK;
}
}  // namespace

int sdg_tensorprod_gradlike_dirXYZ(double* ox, double* oy, double* oz, const double* Mat,
                                   const double* Mat_tr, const double* in, int Nq, int nelem) {
  SDG_TRY(check_order(Nq));
  if (nelem < 0) return fail(SDG_ERR_INVALID_ARG, "nelem < 0");
  if (nelem == 0) return SDG_OK;
  if (!ox || !oy || !oz || !Mat || !Mat_tr || !in)
    return fail(SDG_ERR_INVALID_ARG, "NULL host pointer");
  const double* ins[1] = {in};
  return host_contract(3, ox, oy, oz, Mat, Mat_tr, ins, 1, Nq, nelem, SDG_OPT_GENERAL);
}

int sdg_tensorprod_divlike_dirXYZ_var5(double* ox, double* oy, double* oz, const double* Mat,
                                       const double* Mat_tr, const double* ix,
                                       const double* iy, const double* iz, int Nq,
                                       int nelem) {
  SDG_TRY(check_order(Nq));
  if (nelem < 0 || nelem > 0x7fffffff / 5) return fail(SDG_ERR_INVALID_ARG, "bad nelem %d", nelem);
  if (nelem == 0) return SDG_OK;
  if (!ox || !oy || !oz || !Mat || !Mat_tr || !ix || !iy || !iz)
    return fail(SDG_ERR_INVALID_ARG, "NULL host pointer");
  const double* ins[3] = {ix, iy, iz};
  return host_contract(1, ox, oy, oz, Mat, Mat_tr, ins, 3, Nq, 5 * nelem, SDG_OPT_OPT1);
}

// element_operation_kernel_matvec_dirX / dirY / dirZ (erb:51-129): one
// direction of the gradlike contraction; dir 1 takes Mat_x, dirs 2 and 3 the
// transposed Mat_y_tr / Mat_z_tr, as the templates do.
int sdg_element_matvec_dir_dev(int dir, double* vec_out, const double* Mat, const double* vec_in,
                               int Nq, int nelem, void* stream) {
  SDG_TRY(check_order(Nq));
  if (dir < 1 || dir > 3) return fail(SDG_ERR_INVALID_ARG, "dir %d not in 1..3", dir);
  if (nelem < 0) return fail(SDG_ERR_INVALID_ARG, "nelem < 0");
  if (nelem == 0) return SDG_OK;
  if (!vec_out || !Mat || !vec_in) return fail(SDG_ERR_INVALID_ARG, "NULL device pointer");
  DivArgs a{dir == 1 ? vec_out : nullptr, dir == 2 ? vec_out : nullptr,
            dir == 3 ? vec_out : nullptr, Mat, Mat, vec_in, nullptr, nullptr, nelem};
  return dropin(Nq - 1, 3, SDG_OPT_GENERAL, &a, as_stream(stream));
}

int sdg_element_matvec_dir(int dir, double* vec_out, const double* Mat, const double* vec_in,
                           int Nq, int nelem) {
  SDG_TRY(check_order(Nq));
  if (dir < 1 || dir > 3) return fail(SDG_ERR_INVALID_ARG, "dir %d not in 1..3", dir);
  if (nelem < 0) return fail(SDG_ERR_INVALID_ARG, "nelem < 0");
  if (nelem == 0) return SDG_OK;
  if (!vec_out || !Mat || !vec_in) return fail(SDG_ERR_INVALID_ARG, "NULL host pointer");
  SDG_TRY(require_device());
  const size_t n = (size_t)Nq * Nq * Nq * nelem, nD = (size_t)Nq * Nq;
  Arena ar;
  const size_t oo = ar.add(8 * n), oM = ar.add(8 * nD), oi = ar.add(8 * n);
  SDG_TRY(ar.alloc());
  SDG_CUDA_TRY(cudaMemcpy(ar.at<void>(oM), Mat, 8 * nD, cudaMemcpyHostToDevice));
  SDG_CUDA_TRY(cudaMemcpy(ar.at<void>(oi), vec_in, 8 * n, cudaMemcpyHostToDevice));
  SDG_TRY(sdg_element_matvec_dir_dev(dir, ar.at<double>(oo), ar.at<double>(oM),
                                     ar.at<double>(oi), Nq, nelem, nullptr));
  SDG_CUDA_TRY(cudaMemcpy(vec_out, ar.at<void>(oo), 8 * n, cudaMemcpyDeviceToHost));
  return SDG_OK;
}

int sdg_tensorprod_Lift_hexahedral_dev(double* out, const double* Lift,
                                       const double* in, int Nq, int nelem,
                                       void* stream) {
  SDG_TRY(check_order(Nq));
  if (nelem < 0) return fail(SDG_ERR_INVALID_ARG, "nelem < 0");
  if (nelem == 0) return SDG_OK;
  if (!out || !Lift || !in) return fail(SDG_ERR_INVALID_ARG, "NULL device pointer");
  DivArgs a{out, nullptr, nullptr, Lift, nullptr, in, nullptr, nullptr, nelem};
  return dropin(Nq - 1, 2, SDG_OPT_GENERAL, &a, as_stream(stream));
}

int sdg_tensorprod_Lift_hexahedral(double* out, const double* Lift,
                                   const double* in, int Nq, int nelem) {
  SDG_TRY(check_order(Nq));
  if (nelem < 0) return fail(SDG_ERR_INVALID_ARG, "nelem < 0");
  if (nelem == 0) return SDG_OK;
  if (!out || !Lift || !in) return fail(SDG_ERR_INVALID_ARG, "NULL host pointer");
  SDG_TRY(require_device());
  const size_t np = (size_t)Nq * Nq * Nq;
  const size_t n = np * nelem, nin = 6 * (size_t)Nq * Nq * nelem, nL = 6 * np;
  Arena ar;
  const size_t oo = ar.add(8 * n), oL = ar.add(8 * nL), oi = ar.add(8 * nin);
  SDG_TRY(ar.alloc());
  SDG_CUDA_TRY(cudaMemcpy(ar.at<void>(oL), Lift, 8 * nL, cudaMemcpyHostToDevice));
  SDG_CUDA_TRY(cudaMemcpy(ar.at<void>(oi), in, 8 * nin, cudaMemcpyHostToDevice));
  DivArgs a{ar.at<double>(oo), nullptr, nullptr, ar.at<double>(oL), nullptr,
            ar.at<double>(oi), nullptr, nullptr, nelem};
  SDG_TRY(dropin(Nq - 1, 2, SDG_OPT_GENERAL, &a, nullptr));
  SDG_CUDA_TRY(cudaMemcpy(out, a.ox, 8 * n, cudaMemcpyDeviceToHost));
  return SDG_OK;
}

int sdg_update_halo_dev(double* f, const int* halo_src_map, int Np, int Ne,
                        int NhaloNode, void* stream) {
  if (Np <= 0 || Ne < 0 || NhaloNode < 0)
    return fail(SDG_ERR_INVALID_ARG, "bad sizes Np=%d Ne=%d NhaloNode=%d", Np, Ne,
                NhaloNode);
  if (NhaloNode == 0) return SDG_OK;
  if (!f || !halo_src_map) return fail(SDG_ERR_INVALID_ARG, "NULL device pointer");
  const long long base = (long long)Np * Ne;
  // sources must be owned DOFs: 1..Np*Ne (mod_mesh.f90:184 only maps there)
  update_halo_kernel<<<grid_for(NhaloNode), 256, 0, as_stream(stream)>>>(
      f, halo_src_map, base, NhaloNode, base, nullptr);
  SDG_CUDA_TRY(cudaGetLastError());
  return SDG_OK;
}

int sdg_rk_stage_dev(double* q, const double* q0, const double* dqdt, int Np,
                     int Ne, int stage, double dt, void* stream) {
  // RK3 SSP coefficients, mod_common.f90:28-30
  static const double rk_a[3] = {0.0, 0.75, 1.0 / 3.0};
  static const double rk_b[3] = {1.0, 0.25, 2.0 / 3.0};
  if (stage < 1 || stage > 3) return fail(SDG_ERR_INVALID_ARG, "stage %d outside 1..3", stage);
  if (Np <= 0 || Ne < 0) return fail(SDG_ERR_INVALID_ARG, "bad sizes");
  if (Ne == 0) return SDG_OK;
  if (!q || !dqdt || (stage > 1 && !q0)) return fail(SDG_ERR_INVALID_ARG, "NULL device pointer");
  const long long n = (long long)Np * Ne;
  rk_kernel<<<grid_for(n), 256, 0, as_stream(stream)>>>(q, q0, dqdt, n, rk_a[stage - 1],
                                                       rk_b[stage - 1], dt);
  SDG_CUDA_TRY(cudaGetLastError());
  return SDG_OK;
}

// ---- the time loop on the reference's arrays ---------------------------------

// Scratch of sdg_advect3d_eq_step_dev, 256-byte aligned pieces: two stage
// states (Np*Ne), the face factors (tP, tM) per face node, the resolved
// gather indices (M, P) per face node, the even-odd tables, and per element
// its Escale when that is one value per direction.
static size_t step_layout(int Nq, long long Ne, size_t off[6]) {
  const long long np = (long long)Nq * Nq * Nq, nft = 6LL * Nq * Nq * Ne;
  const int N = Nq, H = N / 2, HR = (N + 1) / 2;
  const long long te = (long long)H * H + (long long)HR * H + (N & 1) * H + HR + H;
  const size_t sizes[6] = {(size_t)(8 * np * Ne), (size_t)(8 * np * Ne), (size_t)(16 * nft),
                           (size_t)(8 * nft), (size_t)(8 * 3 * te), (size_t)(32 * Ne)};
  size_t total = 0;
  for (int k = 0; k < 6; k++) {
    off[k] = total;
    total += (sizes[k] + 255) & ~size_t(255);
  }
  return total;
}

size_t sdg_advect3d_eq_step_scratch_bytes(int Nq, int Ne) {
  if (Nq - 1 < 1 || Nq - 1 > kMaxOrder || Ne < 0) return 0;
  size_t off[6];
  return step_layout(Nq, Ne, off);
}

int sdg_advect3d_eq_step_dev(double* q, const double* u, const double* v, const double* w,
                             const double* D1D, const double* D1D_tr, const double* Lift_mat,
                             const int* VMapM, const int* VMapP, const double* normal_fn,
                             const double* Escale, const double* Fscale,
                             const int* halo_src_map, int Nq, int Np, int NfpTot, int Ne,
                             int NeA, int NhaloNode, double dt, int nstep, int opt,
                             void* scratch, size_t scratch_bytes, int* err_flag,
                             void* stream) {
  // RK3 SSP coefficients, mod_common.f90:28-30
  static const double rk_a[3] = {0.0, 0.75, 1.0 / 3.0};
  static const double rk_b[3] = {1.0, 0.25, 2.0 / 3.0};
  SDG_TRY(check_opt(opt));
  SDG_TRY(check_tend_shape(Nq, Np, NfpTot, Ne, NeA));
  if (nstep < 0 || NhaloNode < 0)
    return fail(SDG_ERR_INVALID_ARG, "nstep %d / NhaloNode %d negative", nstep, NhaloNode);
  if ((long long)Np * NeA > 0x7fffffffLL)
    return fail(SDG_ERR_INVALID_ARG, "Np*NeA beyond the 32-bit DOF ids of VMapM/VMapP");
  if (Ne == 0 || nstep == 0) return SDG_OK;
  size_t off[6];
  const size_t need = step_layout(Nq, Ne, off);
  if (!scratch || scratch_bytes < need)
    return fail(SDG_ERR_INVALID_ARG, "scratch of %zu bytes, %zu needed "
                "(sdg_advect3d_eq_step_scratch_bytes)", scratch_bytes, need);
  if (!q || !u || !v || !w || !D1D || !D1D_tr || !Lift_mat || !VMapM || !VMapP ||
      !normal_fn || !Escale || !Fscale || !err_flag || (NhaloNode > 0 && !halo_src_map))
    return fail(SDG_ERR_INVALID_ARG, "NULL device pointer");
  if ((reinterpret_cast<uintptr_t>(scratch) & 255) != 0)
    return fail(SDG_ERR_INVALID_ARG, "scratch must be 256-byte aligned");
  cudaStream_t st = as_stream(stream);
  char* base = static_cast<char*>(scratch);
  double* qB = reinterpret_cast<double*>(base + off[0]);
  double* qC = reinterpret_cast<double*>(base + off[1]);
  const long long np = Np, nft = (long long)NfpTot * Ne, npne = np * Ne;
  const int p = Nq - 1;

  if (opt != SDG_OPT_EVENODD) {
    // the reference's own sequence and summation order: q0 = q, then per
    // stage update_halo(q), cal_tend into dqdt, the RK update (main.f90:51-80)
    double* flux = reinterpret_cast<double*>(base + off[2]);
    TendArgs ta{qC, q, u, v, w, D1D, D1D_tr, Lift_mat, VMapM, VMapP, normal_fn,
                Escale, Fscale, flux, err_flag, Ne, np * NeA};
    for (int s = 0; s < nstep; s++) {
      SDG_CUDA_TRY(cudaMemcpyAsync(qB, q, 8 * npne, cudaMemcpyDeviceToDevice, st));
      for (int stage = 0; stage < 3; stage++) {
        if (NhaloNode > 0) {
          update_halo_kernel<<<grid_for(NhaloNode), 256, 0, st>>>(q, halo_src_map, npne,
                                                                 NhaloNode, npne, err_flag);
          SDG_CUDA_TRY(cudaGetLastError());
        }
        SDG_TRY(tend_dev(ta, p, NfpTot, opt, st));
        rk_kernel<<<grid_for(npne), 256, 0, st>>>(q, qB, qC, npne, rk_a[stage], rk_b[stage],
                                                   dt);
        SDG_CUDA_TRY(cudaGetLastError());
      }
    }
    // leave the halo slots of q consistent with the final state
    if (NhaloNode > 0) {
      update_halo_kernel<<<grid_for(NhaloNode), 256, 0, st>>>(q, halo_src_map, npne, NhaloNode,
                                                             npne, err_flag);
      SDG_CUDA_TRY(cudaGetLastError());
    }
    return SDG_OK;
  }

  // even-odd: the per-call face data, then one fused launch per stage on
  // ping-pong buffers
  double2* fc = reinterpret_cast<double2*>(base + off[2]);
  int2* res = reinterpret_cast<int2*>(base + off[3]);
  double* tab = reinterpret_cast<double*>(base + off[4]);
  double4* esu = reinterpret_cast<double4*>(base + off[5]);
  StepTablesArgs tb{D1D, D1D_tr, Lift_mat, tab, err_flag};
  SDG_TRY(dropin(p, 5, opt, &tb, st));
  step_face_kernel<<<grid_for(nft), 256, 0, st>>>(VMapM, VMapP, halo_src_map, u, v, w,
                                                  normal_fn, Fscale, res, fc, nft, npne,
                                                  np * NeA, NhaloNode, err_flag);
  SDG_CUDA_TRY(cudaGetLastError());
  step_escale_kernel<<<grid_for(32LL * Ne), 256, 0, st>>>(Escale, esu, Ne, Np);
  SDG_CUDA_TRY(cudaGetLastError());
  StepRefArgs a{};
  a.esu = esu;
  a.u = u;
  a.v = v;
  a.w = w;
  a.tab = tab;
  a.res = res;
  a.fc = fc;
  a.Escale = Escale;
  a.Ne = Ne;
  for (int s = 0; s < nstep; s++) {
    // stage 1: q -> B; 2: B, q0 = q -> C; 3: C, q0 = q -> q
    const double* ins[3] = {q, qB, qC};
    double* outs[3] = {qB, qC, q};
    for (int stage = 0; stage < 3; stage++) {
      a.q_in = ins[stage];
      a.q0 = q;
      a.q_out = outs[stage];
      a.a = rk_a[stage];
      a.b = rk_b[stage];
      a.c = -rk_b[stage] * dt;
      a.rk = stage == 0 ? kRkFirst : kRkGeneral;
      SDG_TRY(dropin(p, 4, opt, &a, st));
    }
  }
  // leave the halo slots of q consistent with the final state
  if (NhaloNode > 0) {
    update_halo_kernel<<<grid_for(NhaloNode), 256, 0, st>>>(q, halo_src_map, npne, NhaloNode,
                                                           npne, err_flag);
    SDG_CUDA_TRY(cudaGetLastError());
  }
  return SDG_OK;
}

}  // extern "C"
