// Device-resident solver for the periodic structured box: state, velocity and
// operators live in HBM; a step is three fused stage launches over rotating
// state buffers (the time loop of main.f90:51-80 without the q0 copy pass and
// without update_halo).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "sdg_df.cuh"
#include "sdg_internal.h"

using namespace sdg;

// One device copy of a solve's buffers, for the pipelined host-to-host path.
struct IoSlot {
  double* q[3] = {nullptr, nullptr, nullptr};
  void* u = nullptr;
  void* v = nullptr;
  void* w = nullptr;
  cudaEvent_t uploaded = nullptr, computed = nullptr, downloaded = nullptr;
};

struct sdg_solver {
  int p = 0, Nq = 0, Np = 0, opt = 0, prec = 0;
  Box box{};
  long long ndof = 0;  // Np * Ne
  cudaStream_t stream = nullptr;
  double* q[3] = {nullptr, nullptr, nullptr};
  int cur = 0;
  void* u = nullptr;
  void* v = nullptr;
  void* w = nullptr;
  void* D = nullptr;
  void* Lift = nullptr;
  double* dqdt = nullptr;
  // face-flux velocity factors shared by the three stages of a step (even-odd
  // FP64 and emulated-FP64 stages; null otherwise): 96 / (p + 1) bytes a DOF.
  // Measured on GB300 against forming them in every stage: 1.04-1.13x for the
  // FP64 stage (p = 7: 19.3 against 18.5 GDOF-updates/s), 1.01-1.14x emulated.
  double* fc = nullptr;
  // elements a stage advances: [elem_begin, elem_begin + elem_count) of the
  // box (the whole box by default; a z-slab partition advances its owned
  // layers and keeps a ghost layer on each side)
  long long elem_begin = 0, elem_count = -1;
  // pipelined host-to-host solves (allocated on first use)
  IoSlot io[2];
  bool io_ready = false;
  cudaStream_t h2d = nullptr, d2h = nullptr, comp = nullptr;
};

namespace {

__global__ void f64_to_f32_kernel(float* out, const double* in, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = (float)in[i];
}

unsigned grid_for(long long n) {
  long long nb = (n + 255) / 256;
  if (nb > 152LL * 64) nb = 152LL * 64;
  return (unsigned)(nb > 0 ? nb : 1);
}

void release(sdg_solver* s) {
  for (IoSlot& io : s->io) {
    for (int i = 0; i < 3; i++) cudaFree(io.q[i]);
    cudaFree(io.u);
    cudaFree(io.v);
    cudaFree(io.w);
    if (io.uploaded) cudaEventDestroy(io.uploaded);
    if (io.computed) cudaEventDestroy(io.computed);
    if (io.downloaded) cudaEventDestroy(io.downloaded);
  }
  if (s->h2d) cudaStreamDestroy(s->h2d);
  if (s->d2h) cudaStreamDestroy(s->d2h);
  if (s->comp) cudaStreamDestroy(s->comp);
  for (int i = 0; i < 3; i++) cudaFree(s->q[i]);
  cudaFree(s->u);
  cudaFree(s->v);
  cudaFree(s->w);
  cudaFree(s->D);
  cudaFree(s->Lift);
  cudaFree(s->dqdt);
  cudaFree(s->fc);
}

// fc: 0 = the stage forms the face-flux velocity factors inline, 1 = it also
// stores them in s->fc, 2 = it reads them from s->fc (an earlier stage of
// the same call, same velocity, stored them); 1 and 2 apply only when s->fc
// exists.
int one_stage_on(sdg_solver* s, int stage, double dt, const double* qin, const double* q0,
                 double* qout, const void* u, const void* v, const void* w, cudaStream_t st,
                 bool tend_only, int fc = 0);

int one_stage(sdg_solver* s, int stage, double dt, const double* qin,
              const double* q0, double* qout, bool tend_only, int fc = 0) {
  return one_stage_on(s, stage, dt, qin, q0, qout, s->u, s->v, s->w, s->stream, tend_only, fc);
}

int one_stage_on(sdg_solver* s, int stage, double dt, const double* qin, const double* q0,
                 double* qout, const void* u, const void* v, const void* w, cudaStream_t st,
                 bool tend_only, int fc) {
  static const double rk_a[3] = {0.0, 0.75, 1.0 / 3.0};  // mod_common.f90:28-30
  static const double rk_b[3] = {1.0, 0.25, 2.0 / 3.0};
  StageArgs a{};
  a.q_in = qin;
  a.q0 = q0;
  a.q_out = qout;
  a.u = u;
  a.v = v;
  a.w = w;
  a.D = s->D;
  a.Lift = s->Lift;
  a.box = s->box;
  a.elem_begin = s->elem_begin;
  a.elem_count = s->elem_count >= 0 ? s->elem_count : s->box.Ne;
  a.a = rk_a[stage];
  a.b = rk_b[stage];
  a.dt = dt;
  const dfl cdt = df_from_double(a.b * dt);
  a.cdt_hi = cdt.hi;
  a.cdt_lo = cdt.lo;
  a.b_is_one = (a.b == 1.0) ? 1 : 0;
  a.a_nonzero = (a.a != 0.0) ? 1 : 0;
  a.tend_only = tend_only ? 1 : 0;
  a.fc_out = (s->fc && fc == 1) ? s->fc : nullptr;
  a.fc_in = (s->fc && fc == 2) ? s->fc : nullptr;
  const double c = tend_only ? 1.0 : a.b * dt;
  for (int d = 0; d < 3; d++) {
    a.eo_sD[d] = -c * s->box.Es[d];
    a.eo_sL[d] = -c * (0.25 * s->box.Fs[d]);
    a.eo_sDf[d] = (float)a.eo_sD[d];
    a.eo_sLf[d] = (float)a.eo_sL[d];
  }
  return launch_stage(s->p, s->prec, s->opt, a, st);
}

// Uploads one velocity component (device source) in the compute type.
int put_velocity(sdg_solver* s, void* dst, const double* src_dev) {
  const long long n = s->ndof;
  if (s->prec != SDG_PREC_FP32) {
    SDG_CUDA_TRY(cudaMemcpyAsync(dst, src_dev, 8 * (size_t)n, cudaMemcpyDeviceToDevice,
                                 s->stream));
  } else {
    f64_to_f32_kernel<<<grid_for(n), 256, 0, s->stream>>>(static_cast<float*>(dst),
                                                         src_dev, n);
    SDG_CUDA_TRY(cudaGetLastError());
  }
  return SDG_OK;
}

// Operator tables in the layout and arithmetic each kernel family reads:
//   FP64: D1D(Nq,Nq) and Lift_mat(Nq,Nq,Nq,6) as given;
//   FP32: the same rounded to float;
//   FP64_EMU: double-float (hi, lo) pairs with the geometric factors folded
//     in: D [3][Nq*Nq] = Es_d*D1D, R [3][Nq] = Es_d * (row sums of D1D, from
//     the FP64 values), Lift [6*Np] = Lift_mat(n,f)*0.5*Fscale(f).
void operator_tables(int prec, int Nq, const Box& box, const double* D1D,
                     const double* Lift_mat, std::vector<unsigned char>& dtab,
                     std::vector<unsigned char>& ltab) {
  const size_t nD = (size_t)Nq * Nq, Np = (size_t)Nq * Nq * Nq, nL = 6 * Np;
  if (prec == SDG_PREC_FP64) {
    dtab.resize(8 * nD);
    ltab.resize(8 * nL);
    std::memcpy(dtab.data(), D1D, 8 * nD);
    std::memcpy(ltab.data(), Lift_mat, 8 * nL);
  } else if (prec == SDG_PREC_FP32) {
    dtab.resize(4 * nD);
    ltab.resize(4 * nL);
    float* d = reinterpret_cast<float*>(dtab.data());
    float* l = reinterpret_cast<float*>(ltab.data());
    for (size_t i = 0; i < nD; i++) d[i] = (float)D1D[i];
    for (size_t i = 0; i < nL; i++) l[i] = (float)Lift_mat[i];
  } else {
    // interleaved double-float pairs: D [3][Nq*Nq], R [3][Nq], Lift [6*Np]
    dtab.resize(8 * (3 * nD + 3 * (size_t)Nq));
    ltab.resize(8 * nL);
    float* d = reinterpret_cast<float*>(dtab.data());
    float* l = reinterpret_cast<float*>(ltab.data());
    for (int ax = 0; ax < 3; ax++) {
      for (size_t i = 0; i < nD; i++) {
        const dfl v = df_from_double(box.Es[ax] * D1D[i]);
        d[2 * (ax * nD + i)] = v.hi;
        d[2 * (ax * nD + i) + 1] = v.lo;
      }
      // true row sums of the FP64 operator (about 1e-16 |D|), in long double
      for (int i = 0; i < Nq; i++) {
        long double rs = 0.0L;
        for (int c = 0; c < Nq; c++) rs += (long double)D1D[i + (size_t)c * Nq];
        const dfl v = df_from_double((double)((long double)box.Es[ax] * rs));
        d[2 * (3 * nD + ax * Nq + i)] = v.hi;
        d[2 * (3 * nD + ax * Nq + i) + 1] = v.lo;
      }
    }
    const int face_axis[6] = {1, 0, 1, 0, 2, 2};  // -y,+x,+y,-x,-z,+z
    for (int f = 0; f < 6; f++)
      for (size_t n = 0; n < Np; n++) {
        const dfl v = df_from_double(Lift_mat[n + f * Np] * (0.5 * box.Fs[face_axis[f]]));
        l[2 * (n + f * Np)] = v.hi;
        l[2 * (n + f * Np) + 1] = v.lo;
      }
  }
}

// Tables of the emulated even-odd stage (sdg_stage_emu_eo.cuh) as
// double-float pairs, per axis: the even-odd tables `eo` (unscaled, from
// eo_tables) with the D parts times -Es_d and the lift parts times
// -0.5*Fs_d, then the row sums R(i), i < N/2, of the symmetrised operator
// (long double) times -Es_d.
void emu_eo_tables(int Nq, const Box& box, const double* D1D, const std::vector<double>& eo,
                   std::vector<unsigned char>& out) {
  const int N = Nq, H = N / 2, HR = (N + 1) / 2, ODD = N & 1;
  const int TE = H * H + HR * H + ODD * H + HR + H, TE2 = TE + H;
  const int offA = H * H + HR * H + ODD * H;
  std::vector<float> f(2 * 3 * (size_t)TE2);
  for (int ax = 0; ax < 3; ax++) {
    const long double sD = -(long double)box.Es[ax];
    const long double sL = -0.5L * (long double)box.Fs[ax];
    auto put = [&](int w, long double v) {
      const dfl x = df_from_double((double)v);
      f[2 * ((size_t)ax * TE2 + w)] = x.hi;
      f[2 * ((size_t)ax * TE2 + w) + 1] = x.lo;
    };
    for (int w = 0; w < TE; w++)
      put(w, (long double)eo[(size_t)ax * TE + w] * (w < offA ? sD : sL));
    for (int i = 0; i < H; i++) {
      long double rs = 0.0L;
      for (int l = 0; l < N; l++)
        rs += 0.5L * ((long double)D1D[i + l * N] - (long double)D1D[(N - 1 - i) + (N - 1 - l) * N]);
      put(TE + i, rs * sD);
    }
  }
  out.resize(4 * f.size());
  std::memcpy(out.data(), f.data(), out.size());
}

// A solver on a given box (sizes and scale factors already checked): the
// operator tables, the state, velocity and face-factor buffers.
int solver_create_box(sdg_solver** out, const Box& box, int p, const double* D1D,
                      const double* Lift_mat, int opt, int precision, void* stream) {
  SDG_TRY(require_device());
  sdg_solver* s = new (std::nothrow) sdg_solver();
  if (!s) return fail(SDG_ERR_OUT_OF_MEMORY, "host allocation failed");
  s->p = p;
  s->Nq = p + 1;
  s->Np = s->Nq * s->Nq * s->Nq;
  s->opt = opt;
  s->prec = precision;
  s->box = box;
  s->ndof = (long long)s->Np * s->box.Ne;
  s->stream = as_stream(stream);
  // velocity element size: FP64 (FP64 and emulated forms) or FP32
  const size_t es = (precision == SDG_PREC_FP32) ? 4 : 8;
  const size_t nD = (size_t)s->Nq * s->Nq, nL = 6 * (size_t)s->Np;
  // operator tables as the kernels read them (see operator_tables below)
  std::vector<unsigned char> dtab, ltab;
  operator_tables(precision, s->Nq, s->box, D1D, Lift_mat, dtab, ltab);
  if (opt == SDG_OPT_EVENODD) {
    std::vector<double> tab;
    const int rc = eo_tables(s->Nq, D1D, Lift_mat, tab);
    if (rc != SDG_OK) {
      delete s;
      return rc;
    }
    if (precision == SDG_PREC_FP64_EMU) {
      emu_eo_tables(s->Nq, s->box, D1D, tab, dtab);
    } else if (precision == SDG_PREC_FP32) {
      // the FP32 form reads FP32 tables
      std::vector<float> f(tab.begin(), tab.end());
      dtab.resize(4 * f.size());
      std::memcpy(dtab.data(), f.data(), dtab.size());
    } else {
      dtab.resize(8 * tab.size());
      std::memcpy(dtab.data(), tab.data(), dtab.size());
    }
  }
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < 3 && e == cudaSuccess; i++)
    e = cudaMalloc(&s->q[i], 8 * (size_t)s->ndof);
  if (e == cudaSuccess) e = cudaMalloc(&s->u, es * (size_t)s->ndof);
  if (e == cudaSuccess) e = cudaMalloc(&s->v, es * (size_t)s->ndof);
  if (e == cudaSuccess) e = cudaMalloc(&s->w, es * (size_t)s->ndof);
  if (e == cudaSuccess) e = cudaMalloc(&s->D, dtab.size());
  if (e == cudaSuccess) e = cudaMalloc(&s->Lift, ltab.size());
  if (e == cudaSuccess && precision != SDG_PREC_FP32 && opt == SDG_OPT_EVENODD)
    e = cudaMalloc(&s->fc, 16 * (size_t)(6 * s->Nq * s->Nq) * (size_t)s->box.Ne);
  if (e == cudaSuccess) e = cudaMemcpy(s->D, dtab.data(), dtab.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(s->Lift, ltab.data(), ltab.size(), cudaMemcpyHostToDevice);
  (void)nD;
  (void)nL;
  if (e != cudaSuccess) {
    const int st = cuda_fail(e, "solver allocation", __FILE__, __LINE__);
    release(s);
    delete s;
    return st;
  }
  *out = s;
  return SDG_OK;
}

}  // namespace

extern "C" {

int sdg_solver_create(sdg_solver** out, int NeX, int NeY, int NeZ, int p,
                      double Lx, double Ly, double Lz, const double* D1D,
                      const double* Lift_mat, int opt, int precision,
                      void* stream) {
  if (!out) return fail(SDG_ERR_INVALID_ARG, "NULL output handle");
  *out = nullptr;
  if (p < 1 || p > kMaxOrder)
    return fail(SDG_ERR_UNSUPPORTED_ORDER, "PolyOrder %d outside 1..15", p);
  if (NeX < 1 || NeY < 1 || NeZ < 1 || !(Lx > 0) || !(Ly > 0) || !(Lz > 0))
    return fail(SDG_ERR_INVALID_ARG, "bad box %dx%dx%d (%g,%g,%g)", NeX, NeY, NeZ,
                Lx, Ly, Lz);
  if ((long long)NeX * NeY * NeZ > 0x7fffffffLL)
    return fail(SDG_ERR_INVALID_ARG, "too many elements");
  if (opt != SDG_OPT_GENERAL && opt != SDG_OPT_OPT1 && opt != SDG_OPT_EVENODD)
    return fail(SDG_ERR_BAD_OPTTYPE, "unknown DGOptrKernel type %d", opt);
  if (precision != SDG_PREC_FP64 && precision != SDG_PREC_FP32 &&
      precision != SDG_PREC_FP64_EMU)
    return fail(SDG_ERR_INVALID_ARG, "unknown precision %d", precision);
  if (!D1D || !Lift_mat) return fail(SDG_ERR_INVALID_ARG, "NULL operator");
  return solver_create_box(out, make_box(NeX, NeY, NeZ, Lx, Ly, Lz), p, D1D, Lift_mat, opt,
                           precision, stream);
}

int sdg_solver_check_mesh(const sdg_solver* s, const int* VMapM, const int* VMapP,
                          const double* normal_fn, const double* Escale,
                          const double* Fscale) {
  if (!s || !VMapM || !VMapP || !normal_fn || !Escale || !Fscale)
    return fail(SDG_ERR_INVALID_ARG, "NULL argument");
  // Rebuild mesh_setup's arrays element by element (mod_mesh.f90:132-190) and
  // compare.  VMapP of a periodic boundary face points at a halo slot; the
  // slot order is the serial loop of mod_mesh.f90:171-190, so it is replayed.
  const int Nq = s->Nq, Np = s->Np, Nfp = Nq * Nq, NfpTot = 6 * Nfp;
  const int NeX = s->box.NeX, NeY = s->box.NeY, NeZ = s->box.NeZ;
  const long long Ne = s->box.Ne, NT = (long long)NfpTot * Ne, NpNe = (long long)Np * Ne;
  const int naxis[6] = {1, 0, 1, 0, 2, 2};
  const double nsign[6] = {-1, 1, 1, -1, -1, 1};
  long long ibuf = 0;
  for (int k = 0; k < NeZ; k++)
    for (int j = 0; j < NeY; j++)
      for (int i = 0; i < NeX; i++) {
        const long long e = i + (long long)NeX * (j + (long long)NeY * k);
        for (int n = 0; n < Np; n++)
          for (int d = 0; d < 3; d++)
            if (Escale[e * Np + n + d * NpNe] != s->box.Es[d])
              return fail(SDG_ERR_MESH, "Escale differs at element %lld node %d", e + 1, n + 1);
        for (int f = 0; f < 6; f++) {
          int ni = i, nj = j, nk = k;
          bool bnd = false;
          switch (f) {
            case 0: bnd = (j == 0); nj = bnd ? NeY - 1 : j - 1; break;
            case 1: bnd = (i == NeX - 1); ni = bnd ? 0 : i + 1; break;
            case 2: bnd = (j == NeY - 1); nj = bnd ? 0 : j + 1; break;
            case 3: bnd = (i == 0); ni = bnd ? NeX - 1 : i - 1; break;
            case 4: bnd = (k == 0); nk = bnd ? NeZ - 1 : k - 1; break;
            default: bnd = (k == NeZ - 1); nk = bnd ? 0 : k + 1; break;
          }
          const long long eP = ni + (long long)NeX * (nj + (long long)NeY * nk);
          for (int fp = 0; fp < Nfp; fp++) {
            const int ta = fp % Nq, tb = fp / Nq, L = Nq - 1, Q2 = Nq * Nq;
            int nM = 0, nP = 0;
            switch (f) {
              case 0: nM = ta + tb * Q2; nP = ta + L * Nq + tb * Q2; break;
              case 1: nM = L + ta * Nq + tb * Q2; nP = ta * Nq + tb * Q2; break;
              case 2: nM = ta + L * Nq + tb * Q2; nP = ta + tb * Q2; break;
              case 3: nM = ta * Nq + tb * Q2; nP = L + ta * Nq + tb * Q2; break;
              case 4: nM = ta + tb * Nq; nP = ta + tb * Nq + L * Q2; break;
              default: nM = ta + tb * Nq + L * Q2; nP = ta + tb * Nq; break;
            }
            const long long m = e * NfpTot + f * Nfp + fp;
            if (VMapM[m] != e * Np + nM + 1)
              return fail(SDG_ERR_MESH, "VMapM differs at face node %lld", m + 1);
            const long long want = bnd ? NpNe + (++ibuf) : eP * Np + nP + 1;
            if (VMapP[m] != want)
              return fail(SDG_ERR_MESH, "VMapP differs at face node %lld", m + 1);
            for (int d = 0; d < 3; d++)
              if (normal_fn[m + d * NT] != (d == naxis[f] ? nsign[f] : 0.0))
                return fail(SDG_ERR_MESH, "normal_fn differs at face node %lld", m + 1);
            if (Fscale[m] != s->box.Fs[naxis[f]])
              return fail(SDG_ERR_MESH, "Fscale differs at face node %lld", m + 1);
          }
        }
      }
  return SDG_OK;
}

int sdg_solver_upload_dev(sdg_solver* s, const double* q, const double* u,
                          const double* v, const double* w) {
  if (!s || !q || !u || !v || !w) return fail(SDG_ERR_INVALID_ARG, "NULL argument");
  SDG_CUDA_TRY(cudaMemcpyAsync(s->q[s->cur], q, 8 * (size_t)s->ndof,
                               cudaMemcpyDeviceToDevice, s->stream));
  SDG_TRY(put_velocity(s, s->u, u));
  SDG_TRY(put_velocity(s, s->v, v));
  SDG_TRY(put_velocity(s, s->w, w));
  return SDG_OK;
}

int sdg_solver_upload(sdg_solver* s, const double* q, const double* u,
                      const double* v, const double* w) {
  if (!s || !q || !u || !v || !w) return fail(SDG_ERR_INVALID_ARG, "NULL argument");
  const size_t bytes = 8 * (size_t)s->ndof;
  SDG_CUDA_TRY(cudaMemcpyAsync(s->q[s->cur], q, bytes, cudaMemcpyHostToDevice, s->stream));
  if (s->prec != SDG_PREC_FP32) {  // FP64 velocity is copied as is
    SDG_CUDA_TRY(cudaMemcpyAsync(s->u, u, bytes, cudaMemcpyHostToDevice, s->stream));
    SDG_CUDA_TRY(cudaMemcpyAsync(s->v, v, bytes, cudaMemcpyHostToDevice, s->stream));
    SDG_CUDA_TRY(cudaMemcpyAsync(s->w, w, bytes, cudaMemcpyHostToDevice, s->stream));
  } else {
    // stage each FP64 component through a free state buffer, then narrow it
    double* tmp = s->q[(s->cur + 1) % 3];
    const double* src[3] = {u, v, w};
    void* dst[3] = {s->u, s->v, s->w};
    for (int c = 0; c < 3; c++) {
      SDG_CUDA_TRY(cudaMemcpyAsync(tmp, src[c], bytes, cudaMemcpyHostToDevice, s->stream));
      SDG_TRY(put_velocity(s, dst[c], tmp));
    }
  }
  return SDG_OK;
}

int sdg_solver_step(sdg_solver* s, double dt, int nstep) {
  if (!s) return fail(SDG_ERR_INVALID_ARG, "NULL solver");
  if (nstep < 0) return fail(SDG_ERR_INVALID_ARG, "nstep < 0");
  for (int it = 0; it < nstep; it++) {
    const int s0 = s->cur, s1 = (s->cur + 1) % 3, s2 = (s->cur + 2) % 3;
    // the velocity cannot change within one call: the first stage of the
    // call forms the face-flux velocity factors and every later stage of the
    // call reads them (a velocity uploaded between calls is formed afresh)
    SDG_TRY(one_stage(s, 0, dt, s->q[s0], nullptr, s->q[s1], false, it == 0 ? 1 : 2));
    SDG_TRY(one_stage(s, 1, dt, s->q[s1], s->q[s0], s->q[s2], false, 2));
    SDG_TRY(one_stage(s, 2, dt, s->q[s2], s->q[s0], s->q[s1], false, 2));
    s->cur = s1;
  }
  return SDG_OK;
}

int sdg_solver_step_timed(sdg_solver* s, double dt, int nstep, double* ms) {
  if (!s || !ms) return fail(SDG_ERR_INVALID_ARG, "NULL argument");
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  SDG_CUDA_TRY(cudaEventCreate(&e0));
  cudaError_t ce = cudaEventCreate(&e1);
  if (ce != cudaSuccess) {
    cudaEventDestroy(e0);
    return cuda_fail(ce, "cudaEventCreate", __FILE__, __LINE__);
  }
  int st = SDG_OK;
  ce = cudaEventRecord(e0, s->stream);
  if (ce == cudaSuccess) st = sdg_solver_step(s, dt, nstep);
  if (ce == cudaSuccess && st == SDG_OK) ce = cudaEventRecord(e1, s->stream);
  if (ce == cudaSuccess && st == SDG_OK) ce = cudaEventSynchronize(e1);
  float f = 0.f;
  if (ce == cudaSuccess && st == SDG_OK) ce = cudaEventElapsedTime(&f, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (ce != cudaSuccess) return cuda_fail(ce, "solver timing", __FILE__, __LINE__);
  if (st != SDG_OK) return st;
  *ms = f;
  return SDG_OK;
}

int sdg_solver_minmax(sdg_solver* s, double* qmin, double* qmax) {
  if (!s || !qmin || !qmax) return fail(SDG_ERR_INVALID_ARG, "NULL argument");
  return sdg_minmax_dev(s->q[s->cur], s->ndof, qmin, qmax, s->stream);
}

// The reference's time loop with its diagnostic output (main.f90:51-80): nstep
// steps, and after every step istep with istep % output_interval == 0 the
// min / max of q over owned DOFs.  The reductions write order keys into a
// device record array on the solver stream, so the loop never waits for the
// host; one copy at the end returns all records.
int sdg_solver_run(sdg_solver* s, double dt, int nstep, int output_interval, double* records) {
  if (!s) return fail(SDG_ERR_INVALID_ARG, "NULL solver");
  if (nstep < 0 || output_interval < 1)
    return fail(SDG_ERR_INVALID_ARG, "nstep < 0 or output_interval < 1");
  const int nout = nstep / output_interval;
  if (nout > 0 && !records) return fail(SDG_ERR_INVALID_ARG, "NULL records");
  unsigned long long* keys = nullptr;
  if (nout > 0)
    SDG_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&keys),
                                 2 * sizeof(unsigned long long) * (size_t)nout, s->stream));
  int rc = SDG_OK;
  for (int k = 0; k < nout && rc == SDG_OK; k++) {
    rc = sdg_solver_step(s, dt, output_interval);
    if (rc == SDG_OK) rc = minmax_launch(s->q[s->cur], s->ndof, keys + 2 * k, keys + 2 * k + 1,
                                         s->stream);
  }
  if (rc == SDG_OK) rc = sdg_solver_step(s, dt, nstep - nout * output_interval);
  std::vector<unsigned long long> hk(2 * (size_t)nout);
  cudaError_t e = cudaSuccess;
  if (rc == SDG_OK && nout > 0)
    e = cudaMemcpyAsync(hk.data(), keys, hk.size() * sizeof(unsigned long long),
                        cudaMemcpyDeviceToHost, s->stream);
  if (keys) cudaFreeAsync(keys, s->stream);
  if (rc != SDG_OK) return rc;
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) return cuda_fail(e, "sdg_solver_run", __FILE__, __LINE__);
  for (size_t i = 0; i < hk.size(); i++) records[i] = minmax_key_to_double(hk[i]);
  return SDG_OK;
}

int sdg_solver_tendency(sdg_solver* s, double* dqdt) {
  if (!s || !dqdt) return fail(SDG_ERR_INVALID_ARG, "NULL argument");
  if (!s->dqdt) SDG_CUDA_TRY(cudaMalloc(&s->dqdt, 8 * (size_t)s->ndof));
  SDG_TRY(one_stage(s, 0, 0.0, s->q[s->cur], nullptr, s->dqdt, true));
  SDG_CUDA_TRY(cudaMemcpyAsync(dqdt, s->dqdt, 8 * (size_t)s->ndof, cudaMemcpyDeviceToHost,
                               s->stream));
  SDG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  return SDG_OK;
}

// Pipelined host-to-host solves: two device buffer sets, an upload stream, a
// compute stream and a download stream, ordered by events so that request
// r+1's upload and request r-1's download overlap request r's kernels.
int sdg_solver_solve_host_pipelined(sdg_solver* s, int count, const double* const* q_in,
                                    const double* const* u, const double* const* v,
                                    const double* const* w, double* const* q_out, double dt,
                                    int nstep) {
  if (!s || count < 0 || nstep < 0 || (count > 0 && (!q_in || !u || !v || !w || !q_out)))
    return fail(SDG_ERR_INVALID_ARG, "bad pipelined solve arguments");
  if (count == 0) return SDG_OK;
  const size_t bytes = 8 * (size_t)s->ndof;
  const size_t es = (s->prec == SDG_PREC_FP32) ? 4 : 8;
  if (!s->io_ready) {
    cudaError_t e = cudaStreamCreateWithFlags(&s->h2d, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->d2h, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->comp, cudaStreamNonBlocking);
    for (IoSlot& io : s->io) {
      for (int i = 0; i < 3 && e == cudaSuccess; i++) e = cudaMalloc(&io.q[i], bytes);
      if (e == cudaSuccess) e = cudaMalloc(&io.u, es * (size_t)s->ndof);
      if (e == cudaSuccess) e = cudaMalloc(&io.v, es * (size_t)s->ndof);
      if (e == cudaSuccess) e = cudaMalloc(&io.w, es * (size_t)s->ndof);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&io.uploaded, cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&io.computed, cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&io.downloaded, cudaEventDisableTiming);
    }
    if (e != cudaSuccess) return cuda_fail(e, "pipelined solve setup", __FILE__, __LINE__);
    s->io_ready = true;
  }
  // the pipeline's work starts after everything already queued on the solver
  cudaEvent_t start;
  SDG_CUDA_TRY(cudaEventCreateWithFlags(&start, cudaEventDisableTiming));
  SDG_CUDA_TRY(cudaEventRecord(start, s->stream));
  SDG_CUDA_TRY(cudaStreamWaitEvent(s->h2d, start, 0));
  cudaEventDestroy(start);
  // A request's result ends in state buffer nstep % 3.  The uploads write
  // buffer 0 (and, in FP32, stage the velocity through a buffer that is not
  // the result), so they wait for the slot's previous download only when the
  // result sits in buffer 0; the compute of a request waits for it always,
  // since the RK stages write every buffer.  The next upload thus overlaps the
  // previous download instead of queueing behind it.
  const int out_buf = nstep % 3;
  const int stage_buf = (out_buf == 1) ? 2 : 1;
  for (int r = 0; r < count; r++) {
    IoSlot& io = s->io[r % 2];
    if (r >= 2) {
      // the slot's previous request must have finished reading its inputs
      SDG_CUDA_TRY(cudaStreamWaitEvent(s->h2d, io.computed, 0));
      if (out_buf == 0) SDG_CUDA_TRY(cudaStreamWaitEvent(s->h2d, io.downloaded, 0));
    }
    SDG_CUDA_TRY(cudaMemcpyAsync(io.q[0], q_in[r], bytes, cudaMemcpyHostToDevice, s->h2d));
    const double* src[3] = {u[r], v[r], w[r]};
    void* dst[3] = {io.u, io.v, io.w};
    for (int c = 0; c < 3; c++) {
      if (s->prec != SDG_PREC_FP32) {
        SDG_CUDA_TRY(cudaMemcpyAsync(dst[c], src[c], bytes, cudaMemcpyHostToDevice, s->h2d));
      } else {
        // FP64 staging through a free state buffer, narrowed on the device
        SDG_CUDA_TRY(cudaMemcpyAsync(io.q[stage_buf], src[c], bytes, cudaMemcpyHostToDevice,
                                     s->h2d));
        f64_to_f32_kernel<<<grid_for(s->ndof), 256, 0, s->h2d>>>(static_cast<float*>(dst[c]),
                                                               io.q[stage_buf], s->ndof);
        SDG_CUDA_TRY(cudaGetLastError());
      }
    }
    SDG_CUDA_TRY(cudaEventRecord(io.uploaded, s->h2d));
    SDG_CUDA_TRY(cudaStreamWaitEvent(s->comp, io.uploaded, 0));
    if (r >= 2) SDG_CUDA_TRY(cudaStreamWaitEvent(s->comp, io.downloaded, 0));
    int cur = 0;
    for (int it = 0; it < nstep; it++) {
      const int s0 = cur, s1 = (cur + 1) % 3, s2 = (cur + 2) % 3;
      SDG_TRY(one_stage_on(s, 0, dt, io.q[s0], nullptr, io.q[s1], io.u, io.v, io.w, s->comp,
                           false, it == 0 ? 1 : 2));
      SDG_TRY(one_stage_on(s, 1, dt, io.q[s1], io.q[s0], io.q[s2], io.u, io.v, io.w, s->comp,
                           false, 2));
      SDG_TRY(one_stage_on(s, 2, dt, io.q[s2], io.q[s0], io.q[s1], io.u, io.v, io.w, s->comp,
                           false, 2));
      cur = s1;
    }
    SDG_CUDA_TRY(cudaEventRecord(io.computed, s->comp));
    SDG_CUDA_TRY(cudaStreamWaitEvent(s->d2h, io.computed, 0));
    SDG_CUDA_TRY(cudaMemcpyAsync(q_out[r], io.q[cur], bytes, cudaMemcpyDeviceToHost, s->d2h));
    SDG_CUDA_TRY(cudaEventRecord(io.downloaded, s->d2h));
  }
  SDG_CUDA_TRY(cudaStreamSynchronize(s->h2d));
  SDG_CUDA_TRY(cudaStreamSynchronize(s->comp));
  SDG_CUDA_TRY(cudaStreamSynchronize(s->d2h));
  return SDG_OK;
}

int sdg_solver_download(sdg_solver* s, double* q) {
  if (!s || !q) return fail(SDG_ERR_INVALID_ARG, "NULL argument");
  SDG_CUDA_TRY(cudaMemcpyAsync(q, s->q[s->cur], 8 * (size_t)s->ndof,
                               cudaMemcpyDeviceToHost, s->stream));
  SDG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  return SDG_OK;
}

const double* sdg_solver_state_dev(const sdg_solver* s) { return s ? s->q[s->cur] : nullptr; }

int sdg_solver_launches_per_step(const sdg_solver* s) { return s ? 3 : 0; }

void* sdg_solver_stream(const sdg_solver* s) { return s ? (void*)s->stream : nullptr; }

int sdg_solver_destroy(sdg_solver* s) {
  if (!s) return SDG_OK;
  release(s);
  delete s;
  return SDG_OK;
}

}  // extern "C"

// ---- z-slab partitions with a face exchange per stage -----------------------
//
// The box is split along z into nparts slabs of whole element layers.  Each
// partition is a solver on its own extended box: its owned layers plus one
// ghost layer below and one above, with the full box's scale factors.  Its
// stages advance only the owned layers; an owned element's -z / +z
// neighbour in the bottom / top layer is then the ghost element, reached
// without the periodic wrap.  Before every stage the partitions exchange the
// face planes the neighbour gathers read -- the bottom owned layer's k = 0
// plane goes to the partition below, the top owned layer's k = Nq-1 plane to
// the one above (periodically) -- through per-partition send and receive
// buffers: pack on the sender, one copy per message, unpack into the
// receiver's own ghost layer.  This is the exchange that update_halo
// (mod_mesh.f90:209-221) stands in for in the single-process reference and
// that MPI carried in SCALE-DG; here the partitions share one GPU, so a
// message is a device-to-device copy (between GPUs it would be a peer copy or
// an NCCL send / receive of the same buffers).  Every owned node computes
// with the same values and factors as in the whole box, so the result equals
// the single-box solver's bit for bit.

struct sdg_slabs {
  int nparts = 0, NeX = 0, NeY = 0, NeZ = 0, Nq = 0, Np = 0;
  std::vector<int> z_begin, lo_src, hi_src;
  std::vector<sdg_solver*> part;
  double* planes = nullptr;  // per partition: send_lo, send_hi, recv_lo, recv_hi
  long long plane_n = 0;     // doubles of one plane: NeX*NeY*Nq^2
  cudaStream_t stream = nullptr;
};

namespace {

// send_lo <- the k = 0 plane of the bottom owned layer (first element lo0);
// send_hi <- the k = Nq-1 plane of the top owned layer (first element hi0).
__global__ void slab_pack_kernel(const double* __restrict__ q, double* send_lo, double* send_hi,
                                 long long lo0, long long hi0, long long n, int Nq) {
  const int nq2 = Nq * Nq;
  const long long np = (long long)nq2 * Nq;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const long long e = t / nq2;
    const int n2 = (int)(t - e * nq2);
    send_lo[t] = q[(lo0 + e) * np + n2];
    send_hi[t] = q[(hi0 + e) * np + (long long)(Nq - 1) * nq2 + n2];
  }
}

// The lower ghost layer (first element g_lo) receives the k = Nq-1 plane its
// upper neighbour reads; the upper ghost layer (g_hi) the k = 0 plane.
__global__ void slab_unpack_kernel(double* q, const double* __restrict__ recv_lo,
                                   const double* __restrict__ recv_hi, long long g_lo,
                                   long long g_hi, long long n, int Nq) {
  const int nq2 = Nq * Nq;
  const long long np = (long long)nq2 * Nq;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const long long e = t / nq2;
    const int n2 = (int)(t - e * nq2);
    q[(g_lo + e) * np + (long long)(Nq - 1) * nq2 + n2] = recv_lo[t];
    q[(g_hi + e) * np + n2] = recv_hi[t];
  }
}

int slab_layers(const sdg_slabs* s, int k) { return s->z_begin[k + 1] - s->z_begin[k]; }

// The exchange before a stage reads state buffer `buf` of every partition.
int slab_exchange(sdg_slabs* s, int buf) {
  const long long nxy = (long long)s->NeX * s->NeY, n = s->plane_n;
  const int P = s->nparts;
  auto plane = [&](int k, int which) { return s->planes + (4LL * k + which) * n; };
  for (int k = 0; k < P; k++) {
    slab_pack_kernel<<<grid_for(n), 256, 0, s->stream>>>(
        s->part[k]->q[buf], plane(k, 0), plane(k, 1), nxy, nxy * slab_layers(s, k), n, s->Nq);
    SDG_CUDA_TRY(cudaGetLastError());
  }
  // messages: partition k's lower ghost plane comes from lo_src[k]'s top
  // layer, its upper one from hi_src[k]'s bottom layer
  for (int k = 0; k < P; k++) {
    SDG_CUDA_TRY(cudaMemcpyAsync(plane(k, 2), plane(s->lo_src[k], 1), 8 * n,
                                 cudaMemcpyDeviceToDevice, s->stream));
    SDG_CUDA_TRY(cudaMemcpyAsync(plane(k, 3), plane(s->hi_src[k], 0), 8 * n,
                                 cudaMemcpyDeviceToDevice, s->stream));
  }
  for (int k = 0; k < P; k++) {
    slab_unpack_kernel<<<grid_for(n), 256, 0, s->stream>>>(
        s->part[k]->q[buf], plane(k, 2), plane(k, 3), 0, nxy * (slab_layers(s, k) + 1), n,
        s->Nq);
    SDG_CUDA_TRY(cudaGetLastError());
  }
  return SDG_OK;
}

// Gathers partition k's extended layers (one ghost layer each side, periodic
// in z) of a whole-box host field.
void slab_extend(const sdg_slabs* s, int k, const double* full, std::vector<double>& out) {
  const long long lay = (long long)s->NeX * s->NeY * s->Np;
  const int nz = slab_layers(s, k);
  out.resize((size_t)(lay * (nz + 2)));
  for (int l = 0; l < nz + 2; l++) {
    const int z = ((s->z_begin[k] - 1 + l) % s->NeZ + s->NeZ) % s->NeZ;
    std::memcpy(out.data() + l * lay, full + z * lay, 8 * (size_t)lay);
  }
}

}  // namespace

extern "C" {

int sdg_slab_plan(int NeZ, int nparts, int* z_begin, int* lo_src, int* hi_src) {
  if (NeZ < 1 || nparts < 1 || nparts > NeZ)
    return fail(SDG_ERR_INVALID_ARG, "cannot split %d element layers into %d slabs", NeZ,
                nparts);
  if (!z_begin || !lo_src || !hi_src) return fail(SDG_ERR_INVALID_ARG, "NULL argument");
  for (int k = 0; k <= nparts; k++) z_begin[k] = (int)((long long)k * NeZ / nparts);
  for (int k = 0; k < nparts; k++) {
    lo_src[k] = (k + nparts - 1) % nparts;
    hi_src[k] = (k + 1) % nparts;
  }
  return SDG_OK;
}

int sdg_slabs_create(sdg_slabs** out, int NeX, int NeY, int NeZ, int p, double Lx, double Ly,
                     double Lz, const double* D1D, const double* Lift_mat, int opt,
                     int precision, int nparts, void* stream) {
  if (!out) return fail(SDG_ERR_INVALID_ARG, "NULL output handle");
  *out = nullptr;
  if (p < 1 || p > kMaxOrder)
    return fail(SDG_ERR_UNSUPPORTED_ORDER, "PolyOrder %d outside 1..15", p);
  if (NeX < 1 || NeY < 1 || NeZ < 1 || !(Lx > 0) || !(Ly > 0) || !(Lz > 0))
    return fail(SDG_ERR_INVALID_ARG, "bad box %dx%dx%d", NeX, NeY, NeZ);
  if (nparts < 1 || nparts > NeZ)
    return fail(SDG_ERR_INVALID_ARG, "cannot split %d element layers into %d slabs", NeZ,
                nparts);
  if ((long long)NeX * NeY * (NeZ + 2LL * nparts) > 0x7fffffffLL)
    return fail(SDG_ERR_INVALID_ARG, "too many elements");
  if (opt != SDG_OPT_GENERAL && opt != SDG_OPT_OPT1 && opt != SDG_OPT_EVENODD)
    return fail(SDG_ERR_BAD_OPTTYPE, "unknown DGOptrKernel type %d", opt);
  if (precision != SDG_PREC_FP64 && precision != SDG_PREC_FP32 &&
      precision != SDG_PREC_FP64_EMU)
    return fail(SDG_ERR_INVALID_ARG, "unknown precision %d", precision);
  if (!D1D || !Lift_mat) return fail(SDG_ERR_INVALID_ARG, "NULL operator");
  sdg_slabs* s = new (std::nothrow) sdg_slabs();
  if (!s) return fail(SDG_ERR_OUT_OF_MEMORY, "host allocation failed");
  s->nparts = nparts;
  s->NeX = NeX;
  s->NeY = NeY;
  s->NeZ = NeZ;
  s->Nq = p + 1;
  s->Np = s->Nq * s->Nq * s->Nq;
  s->stream = as_stream(stream);
  s->z_begin.resize(nparts + 1);
  s->lo_src.resize(nparts);
  s->hi_src.resize(nparts);
  int st = sdg_slab_plan(NeZ, nparts, s->z_begin.data(), s->lo_src.data(), s->hi_src.data());
  if (st != SDG_OK) {
    delete s;
    return st;
  }
  const Box full = make_box(NeX, NeY, NeZ, Lx, Ly, Lz);
  const long long nxy = (long long)NeX * NeY;
  for (int k = 0; k < nparts && st == SDG_OK; k++) {
    Box b = full;  // the whole box's scale factors, bit for bit
    b.NeZ = slab_layers(s, k) + 2;
    b.Ne = nxy * b.NeZ;
    sdg_solver* ps = nullptr;
    st = solver_create_box(&ps, b, p, D1D, Lift_mat, opt, precision, stream);
    if (st == SDG_OK) {
      ps->elem_begin = nxy;
      ps->elem_count = nxy * slab_layers(s, k);
      s->part.push_back(ps);
    }
  }
  s->plane_n = nxy * s->Nq * s->Nq;
  if (st == SDG_OK) {
    const cudaError_t e = cudaMalloc(&s->planes, 8 * 4 * (size_t)nparts * (size_t)s->plane_n);
    if (e != cudaSuccess) st = cuda_fail(e, "slab planes", __FILE__, __LINE__);
  }
  if (st != SDG_OK) {
    sdg_slabs_destroy(s);
    return st;
  }
  *out = s;
  return SDG_OK;
}

int sdg_slabs_upload(sdg_slabs* s, const double* q, const double* u, const double* v,
                     const double* w) {
  if (!s || !q || !u || !v || !w) return fail(SDG_ERR_INVALID_ARG, "NULL argument");
  std::vector<double> eq, eu, ev, ew;
  for (int k = 0; k < s->nparts; k++) {
    slab_extend(s, k, q, eq);
    slab_extend(s, k, u, eu);
    slab_extend(s, k, v, ev);
    slab_extend(s, k, w, ew);
    SDG_TRY(sdg_solver_upload(s->part[k], eq.data(), eu.data(), ev.data(), ew.data()));
    // the host vectors are reused for the next partition: let the copies land
    SDG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  }
  return SDG_OK;
}

int sdg_slabs_step(sdg_slabs* s, double dt, int nstep) {
  if (!s) return fail(SDG_ERR_INVALID_ARG, "NULL slabs");
  if (nstep < 0) return fail(SDG_ERR_INVALID_ARG, "nstep < 0");
  for (int it = 0; it < nstep; it++) {
    const int s0 = s->part[0]->cur, s1 = (s0 + 1) % 3, s2 = (s0 + 2) % 3;
    SDG_TRY(slab_exchange(s, s0));
    for (sdg_solver* ps : s->part)
      SDG_TRY(one_stage(ps, 0, dt, ps->q[s0], nullptr, ps->q[s1], false, it == 0 ? 1 : 2));
    SDG_TRY(slab_exchange(s, s1));
    for (sdg_solver* ps : s->part)
      SDG_TRY(one_stage(ps, 1, dt, ps->q[s1], ps->q[s0], ps->q[s2], false, 2));
    SDG_TRY(slab_exchange(s, s2));
    for (sdg_solver* ps : s->part)
      SDG_TRY(one_stage(ps, 2, dt, ps->q[s2], ps->q[s0], ps->q[s1], false, 2));
    for (sdg_solver* ps : s->part) ps->cur = s1;
  }
  return SDG_OK;
}

int sdg_slabs_download(sdg_slabs* s, double* q) {
  if (!s || !q) return fail(SDG_ERR_INVALID_ARG, "NULL argument");
  const long long lay = (long long)s->NeX * s->NeY * s->Np;
  for (int k = 0; k < s->nparts; k++) {
    const sdg_solver* ps = s->part[k];
    SDG_CUDA_TRY(cudaMemcpyAsync(q + s->z_begin[k] * lay, ps->q[ps->cur] + lay,
                                 8 * (size_t)(lay * slab_layers(s, k)), cudaMemcpyDeviceToHost,
                                 s->stream));
  }
  SDG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  return SDG_OK;
}

long long sdg_slabs_exchange_bytes(const sdg_slabs* s) {
  return s ? 8LL * 2 * s->nparts * s->plane_n : 0;
}

int sdg_slabs_destroy(sdg_slabs* s) {
  if (!s) return SDG_OK;
  if (s->stream) cudaStreamSynchronize(s->stream);
  for (sdg_solver* ps : s->part) sdg_solver_destroy(ps);
  cudaFree(s->planes);
  delete s;
  return SDG_OK;
}

}  // extern "C"
