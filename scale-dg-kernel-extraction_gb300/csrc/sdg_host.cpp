// Host-side parts of libsdg_gb300: status reporting, operator data (file
// reader and generator), the DGOptrKernel type switch, and small helpers.
#include <cuda_runtime.h>

#include <atomic>
#include <cctype>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "sdg_internal.h"

namespace sdg {

static thread_local std::string g_last_error;

int fail(int status, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return status;
}

int cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
  const int st = (e == cudaErrorMemoryAllocation) ? SDG_ERR_OUT_OF_MEMORY
               : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
                   ? SDG_ERR_NO_DEVICE
                   : SDG_ERR_CUDA;
  return fail(st, "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file,
              line);
}

int set_kernel_smem(const void* func, int smem, bool max_carveout) {
  int dev = 0;
  SDG_CUDA_TRY(cudaGetDevice(&dev));
  struct Key {
    const void* func;
    int dev, smem;
    bool carve;
    bool operator==(const Key& o) const {
      return func == o.func && dev == o.dev && smem == o.smem && carve == o.carve;
    }
  };
  static std::mutex mu;
  static std::vector<Key> done;  // a few dozen kernels at most
  const Key k{func, dev, smem, max_carveout};
  {
    std::lock_guard<std::mutex> g(mu);
    if (std::find(done.begin(), done.end(), k) != done.end()) return SDG_OK;
  }
  SDG_CUDA_TRY(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  if (max_carveout)
    SDG_CUDA_TRY(cudaFuncSetAttribute(func, cudaFuncAttributePreferredSharedMemoryCarveout,
                                      (int)cudaSharedmemCarveoutMaxShared));
  std::lock_guard<std::mutex> g(mu);
  if (std::find(done.begin(), done.end(), k) == done.end()) done.push_back(k);
  return SDG_OK;
}

int require_device() {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    return fail(SDG_ERR_NO_DEVICE, "no CUDA device is visible (%s)",
                cudaGetErrorString(e));
  }
  return SDG_OK;
}

Box make_box(int NeX, int NeY, int NeZ, double Lx, double Ly, double Lz) {
  Box b;
  b.NeX = NeX;
  b.NeY = NeY;
  b.NeZ = NeZ;
  b.Ne = (long long)NeX * NeY * NeZ;
  // dx = domsize / real(NeX) and 2/dx, mod_mesh.f90:112-114, :147-149, :369-394
  const double dx = Lx / (double)NeX, dy = Ly / (double)NeY,
               dz = Lz / (double)NeZ;
  b.Es[0] = 2.0 / dx;
  b.Es[1] = 2.0 / dy;
  b.Es[2] = 2.0 / dz;
  for (int d = 0; d < 3; d++) {
    b.Fs[d] = b.Es[d];
    b.Esf[d] = (float)b.Es[d];
    b.hFsf[d] = (float)(0.5 * b.Fs[d]);
  }
  return b;
}

// ---------------------------------------------------------------------------
// Operator file reader: the three list-directed reads of element_init
// (mod_mesh.f90:253-261).  Each read starts on a new record and skips what is
// left of the last record it used.  Separators: blanks, commas, line ends;
// exponent letter E or D; "r*c" repeat counts.
namespace {
struct ListReader {
  const std::string& s;
  size_t pos = 0;
  explicit ListReader(const std::string& str) : s(str) {}
  bool read(double* out, long n) {
    long got = 0;
    size_t p = pos;
    while (got < n) {
      while (p < s.size() && (s[p] == ' ' || s[p] == '\t' || s[p] == ',' ||
                              s[p] == '\n' || s[p] == '\r'))
        p++;
      if (p >= s.size() || s[p] == '/') return false;
      std::string tok;
      while (p < s.size() && !std::isspace((unsigned char)s[p]) &&
             s[p] != ',' && s[p] != '/') {
        char c = s[p++];
        tok.push_back((c == 'D' || c == 'd') ? 'E' : c);
        if (tok.size() > 100) return false;
      }
      long rep = 1;
      std::string val = tok;
      const size_t star = tok.find('*');
      if (star != std::string::npos) {
        char* end = nullptr;
        rep = std::strtol(tok.substr(0, star).c_str(), &end, 10);
        if (!end || *end != '\0' || rep <= 0) return false;
        val = tok.substr(star + 1);
      }
      char* end = nullptr;
      const double x = std::strtod(val.c_str(), &end);
      if (end == val.c_str() || *end != '\0') return false;
      for (long r = 0; r < rep && got < n; r++) out[got++] = x;
    }
    while (p < s.size() && s[p] != '\n') p++;
    if (p < s.size()) p++;
    pos = p;
    return true;
  }
};
}  // namespace

// ---------------------------------------------------------------------------
// Operator generator.  Gauss-Lobatto-Legendre nodes of degree N are -1, 1
// and the roots of P_N'; they are found by Newton iteration on
// (1 - x^2) P_N'(x) written through the Legendre recurrence, started from the
// Chebyshev-Gauss-Lobatto points, in long double.  The Lagrange
// differentiation matrix on these nodes is
//   D_ij = P_N(x_i) / (P_N(x_j) (x_i - x_j))   (i != j),
//   D_00 = -N(N+1)/4,  D_NN = N(N+1)/4,  D_ii = 0 otherwise.
// With the exact (non-lumped) mass matrix M = (V V^T)^{-1}, V_in = Ptilde_n(x_i)
// the orthonormal Legendre Vandermonde, the lift of a face is
// M^{-1} e_face = V V^T e_face in the face-normal direction and the identity
// across the face, so Lift(i,j,k,f) is a function of the normal index only:
//   c_minus(m) = sum_n (2n+1)/2 P_n(x_m) (-1)^n,  c_plus(m) = sum_n (2n+1)/2 P_n(x_m).
namespace {
void legendre_all(int N, long double x, long double* P) {
  P[0] = 1.0L;
  if (N >= 1) P[1] = x;
  for (int n = 2; n <= N; n++)
    P[n] = ((2.0L * n - 1.0L) * x * P[n - 1] - (n - 1.0L) * P[n - 2]) / n;
}

void gll_nodes(int N, long double* x) {
  const long double pi = 3.141592653589793238462643383279502884L;
  std::vector<long double> P(N + 1);
  for (int j = 0; j <= N; j++) {
    // ascending order: x_0 = -1 ... x_N = 1
    long double xi = -std::cos(pi * (long double)j / (long double)N);
    for (int it = 0; it < 100; it++) {
      legendre_all(N, xi, P.data());
      const long double dxi = (xi * P[N] - P[N - 1]) / ((N + 1) * P[N]);
      xi -= dxi;
      if (std::fabs(dxi) < 1e-30L) break;
    }
    x[j] = xi;
  }
  x[0] = -1.0L;
  x[N] = 1.0L;
  // the nodes are symmetric: enforce it exactly
  for (int j = 0; j <= N / 2; j++) {
    const long double s = 0.5L * (x[N - j] - x[j]);
    x[j] = -s;
    x[N - j] = s;
  }
  if (N % 2 == 0) x[N / 2] = 0.0L;
}
}  // namespace

// Tables of the even-odd stage bodies (sdg_stage_eo.cuh), per direction x, y,
// z: E(i,l), O(i,l), D(i,mid) from the centro-antisymmetric part of D1D and
// A(i), B(i) from the face lift columns.  Checks, relative to max|D| and
// max|Lift|, that D1D is centro-antisymmetric, that each face's lift is a
// column along the normal constant over the tangential nodes and that the +
// face's column mirrors the - face's, all within 1e-13 (the operator files
// hold them to 2.4e-14 at p = 15), then builds the tables from the
// symmetrised operators in long double.
int eo_tables(int Nq, const double* D1D, const double* Lift_mat, std::vector<double>& tab) {
  const int N = Nq, H = N / 2, HR = (N + 1) / 2, ODD = N & 1;
  const int TE = H * H + HR * H + ODD * H + HR + H;
  const long long Np = (long long)N * N * N;
  const double tol = 1e-13;
  double maxD = 0.0, maxL = 0.0;
  for (int i = 0; i < N * N; i++) maxD = std::fmax(maxD, std::fabs(D1D[i]));
  for (long long i = 0; i < 6 * Np; i++) maxL = std::fmax(maxL, std::fabs(Lift_mat[i]));
  auto D = [&](int i, int l) { return (long double)D1D[i + l * N]; };
  for (int i = 0; i < N; i++)
    for (int l = 0; l < N; l++)
      if (std::fabs(D1D[i + l * N] + D1D[(N - 1 - i) + (N - 1 - l) * N]) > tol * maxD)
        return fail(SDG_ERR_INVALID_ARG,
                    "D1D is not centro-antisymmetric (entry %d,%d); use SDG_OPT_OPT1", i, l);
  // lift column of face f along its normal: mean over the tangential nodes
  const int fminus[3] = {3, 0, 4}, fplus[3] = {1, 2, 5};
  auto node = [&](int ax, int m, int t1, int t2) {
    // normal index m on axis ax, tangential indices on the other two axes
    int c[3];
    c[ax] = m;
    c[(ax + 1) % 3] = t1;
    c[(ax + 2) % 3] = t2;
    return c[0] + (long long)c[1] * N + (long long)c[2] * N * N;
  };
  std::vector<long double> col(2 * (size_t)N);
  tab.assign(3 * (size_t)TE, 0.0);
  for (int ax = 0; ax < 3; ax++) {
    for (int side = 0; side < 2; side++) {
      const int f = side ? fplus[ax] : fminus[ax];
      for (int m = 0; m < N; m++) {
        long double sum = 0.0L;
        for (int t1 = 0; t1 < N; t1++)
          for (int t2 = 0; t2 < N; t2++) sum += Lift_mat[node(ax, m, t1, t2) + f * Np];
        const long double mean = sum / ((long double)N * N);
        for (int t1 = 0; t1 < N; t1++)
          for (int t2 = 0; t2 < N; t2++)
            if (std::fabs((double)(Lift_mat[node(ax, m, t1, t2) + f * Np] - mean)) > tol * maxL)
              return fail(SDG_ERR_INVALID_ARG,
                          "Lift_mat face %d is not separable; use SDG_OPT_OPT1", f + 1);
        col[side * N + m] = mean;
      }
    }
    for (int m = 0; m < N; m++)
      if (std::fabs((double)(col[m] - col[N + (N - 1 - m)])) > tol * maxL)
        return fail(SDG_ERR_INVALID_ARG,
                    "Lift_mat faces %d/%d are not mirror images; use SDG_OPT_OPT1",
                    fminus[ax] + 1, fplus[ax] + 1);
    double* T = tab.data() + (size_t)ax * TE;
    auto Ds = [&](int i, int l) { return 0.5L * (D(i, l) - D(N - 1 - i, N - 1 - l)); };
    for (int i = 0; i < H; i++)
      for (int l = 0; l < H; l++) T[i * H + l] = (double)(0.5L * (Ds(i, l) + Ds(i, N - 1 - l)));
    for (int i = 0; i < HR; i++)
      for (int l = 0; l < H; l++)
        T[H * H + i * H + l] = (double)(0.5L * (Ds(i, l) - Ds(i, N - 1 - l)));
    if (ODD)
      for (int i = 0; i < H; i++) T[H * H + HR * H + i] = (double)Ds(i, H);
    // symmetrised minus-face column lam(m); the plus face is lam(N-1-m)
    auto lam = [&](int m) { return 0.5L * (col[m] + col[N + (N - 1 - m)]); };
    const int oA = H * H + HR * H + ODD * H, oB = oA + HR;
    for (int i = 0; i < HR; i++) T[oA + i] = (double)(0.5L * (lam(i) + lam(N - 1 - i)));
    for (int i = 0; i < H; i++) T[oB + i] = (double)(0.5L * (lam(i) - lam(N - 1 - i)));
  }
  return SDG_OK;
}


}  // namespace sdg

using namespace sdg;

extern "C" {

const char* sdg_status_string(int status) {
  switch (status) {
    case SDG_OK: return "ok";
    case SDG_ERR_INVALID_ARG: return "invalid argument";
    case SDG_ERR_UNSUPPORTED_ORDER: return "unsupported polynomial order (1..15)";
    case SDG_ERR_BAD_OPTTYPE: return "unsupported DGOptrKernel type";
    case SDG_ERR_CUDA: return "CUDA error";
    case SDG_ERR_OUT_OF_MEMORY: return "out of memory";
    case SDG_ERR_FILE: return "operator file missing or malformed";
    case SDG_ERR_MESH: return "mesh index out of range or mesh mismatch";
    case SDG_ERR_TIMEOUT: return "bounded wait expired";
    case SDG_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown status";
  }
}

const char* sdg_last_error(void) { return g_last_error.c_str(); }

const char* sdg_version(void) { return "sdg_gb300 0.1 (sm_103a)"; }

size_t sdg_struct_size(const char* name) {
  if (!name) return 0;
  const std::string n(name);
  if (n == "sdg_server_config") return sizeof(sdg_server_config);
  if (n == "sdg_request") return sizeof(sdg_request);
  if (n == "sdg_result") return sizeof(sdg_result);
  if (n == "sdg_server_stats") return sizeof(sdg_server_stats);
  return 0;
}

int sdg_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

int sdg_set_device(int device) {
  SDG_TRY(require_device());
  SDG_CUDA_TRY(cudaSetDevice(device));
  return SDG_OK;
}

int sdg_device_synchronize(void) {
  SDG_TRY(require_device());
  SDG_CUDA_TRY(cudaDeviceSynchronize());
  return SDG_OK;
}

int sdg_dev_alloc(size_t bytes, void** out) {
  if (!out) return fail(SDG_ERR_INVALID_ARG, "NULL output pointer");
  *out = nullptr;
  SDG_TRY(require_device());
  SDG_CUDA_TRY(cudaMalloc(out, bytes ? bytes : 1));
  return SDG_OK;
}

int sdg_dev_free(void* p) {
  if (!p) return SDG_OK;
  SDG_CUDA_TRY(cudaFree(p));
  return SDG_OK;
}

int sdg_memcpy_h2d(void* dst, const void* src, size_t bytes) {
  if (!bytes) return SDG_OK;
  if (!dst || !src) return fail(SDG_ERR_INVALID_ARG, "NULL pointer");
  SDG_CUDA_TRY(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
  return SDG_OK;
}

int sdg_memcpy_d2h(void* dst, const void* src, size_t bytes) {
  if (!bytes) return SDG_OK;
  if (!dst || !src) return fail(SDG_ERR_INVALID_ARG, "NULL pointer");
  SDG_CUDA_TRY(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
  return SDG_OK;
}

int sdg_memcpy_d2d_async(void* dst, const void* src, size_t bytes, void* stream) {
  if (!bytes) return SDG_OK;
  if (!dst || !src) return fail(SDG_ERR_INVALID_ARG, "NULL pointer");
  SDG_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, as_stream(stream)));
  return SDG_OK;
}

int sdg_memset_dev(void* dst, int value, size_t bytes) {
  if (!bytes) return SDG_OK;
  if (!dst) return fail(SDG_ERR_INVALID_ARG, "NULL pointer");
  SDG_CUDA_TRY(cudaMemset(dst, value, bytes));
  return SDG_OK;
}

int sdg_pinned_alloc(size_t bytes, void** out) {
  if (!out) return fail(SDG_ERR_INVALID_ARG, "NULL output pointer");
  *out = nullptr;
  SDG_TRY(require_device());
  SDG_CUDA_TRY(cudaHostAlloc(out, bytes ? bytes : 1, cudaHostAllocDefault));
  return SDG_OK;
}

int sdg_pinned_free(void* p) {
  if (!p) return SDG_OK;
  SDG_CUDA_TRY(cudaFreeHost(p));
  return SDG_OK;
}

int sdg_operator_read(const char* path, int p, double* x1D, double* D1D,
                      double* D1D_tr, double* Lift_mat) {
  if (p < 1 || p > kMaxOrder)
    return fail(SDG_ERR_UNSUPPORTED_ORDER, "PolyOrder %d outside 1..%d", p,
                kMaxOrder);
  if (!path || !x1D || !D1D || !Lift_mat)
    return fail(SDG_ERR_INVALID_ARG, "NULL argument");
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(SDG_ERR_FILE, "cannot open operator file %s", path);
  std::string s;
  char buf[1 << 16];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) s.append(buf, n);
  std::fclose(f);
  const int Nq = p + 1;
  ListReader r(s);
  if (!r.read(x1D, Nq) || !r.read(D1D, (long)Nq * Nq) ||
      !r.read(Lift_mat, 6L * Nq * Nq * Nq))
    return fail(SDG_ERR_FILE, "operator file %s is short or malformed for p=%d",
                path, p);
  if (D1D_tr)
    for (int j = 0; j < Nq; j++)
      for (int i = 0; i < Nq; i++) D1D_tr[i + j * Nq] = D1D[j + i * Nq];
  return SDG_OK;
}

int sdg_operator_generate(int p, double* x1D, double* D1D, double* D1D_tr,
                          double* Lift_mat) {
  if (p < 1 || p > kMaxOrder)
    return fail(SDG_ERR_UNSUPPORTED_ORDER, "PolyOrder %d outside 1..%d", p,
                kMaxOrder);
  if (!x1D || !D1D || !Lift_mat) return fail(SDG_ERR_INVALID_ARG, "NULL argument");
  const int N = p, Nq = p + 1;
  std::vector<long double> x(Nq), PN(Nq), P(Nq);
  gll_nodes(N, x.data());
  for (int i = 0; i < Nq; i++) {
    legendre_all(N, x[i], P.data());
    PN[i] = P[N];
    x1D[i] = (double)x[i];
  }
  for (int j = 0; j < Nq; j++)
    for (int i = 0; i < Nq; i++) {
      long double d;
      if (i != j) d = PN[i] / (PN[j] * (x[i] - x[j]));
      else if (i == 0) d = -(long double)(N * (N + 1)) / 4.0L;
      else if (i == N) d = (long double)(N * (N + 1)) / 4.0L;
      else d = 0.0L;
      D1D[i + j * Nq] = (double)d;
    }
  if (D1D_tr)
    for (int j = 0; j < Nq; j++)
      for (int i = 0; i < Nq; i++) D1D_tr[i + j * Nq] = D1D[j + i * Nq];
  std::vector<double> cm(Nq), cp(Nq);
  for (int m = 0; m < Nq; m++) {
    legendre_all(N, x[m], P.data());
    long double sm = 0.0L, sp = 0.0L;
    for (int n = 0; n <= N; n++) {
      const long double wn = (2.0L * n + 1.0L) / 2.0L * P[n];
      sp += wn;
      sm += (n % 2 ? -wn : wn);
    }
    cm[m] = (double)sm;
    cp[m] = (double)sp;
  }
  const long Np = (long)Nq * Nq * Nq;
  for (int k = 0; k < Nq; k++)
    for (int j = 0; j < Nq; j++)
      for (int i = 0; i < Nq; i++) {
        const long nidx = i + (long)j * Nq + (long)k * Nq * Nq;
        Lift_mat[nidx + 0 * Np] = cm[j];  // face 1: -y
        Lift_mat[nidx + 1 * Np] = cp[i];  // face 2: +x
        Lift_mat[nidx + 2 * Np] = cp[j];  // face 3: +y
        Lift_mat[nidx + 3 * Np] = cm[i];  // face 4: -x
        Lift_mat[nidx + 4 * Np] = cm[k];  // face 5: -z
        Lift_mat[nidx + 5 * Np] = cp[k];  // face 6: +z
      }
  return SDG_OK;
}

// dg_optr_kernel_setup, mod_dg_optr_kernel.f90:45-58.  The reference keeps the
// choice in the module variable eval_typeid; this is its process-wide mirror.
static std::atomic<int> g_opttype{0};

int sdg_dg_optr_kernel_setup(const char* t) {
  if (!t) return fail(SDG_ERR_INVALID_ARG, "NULL DGOptrKernel type");
  std::string s(t);
  while (!s.empty() && s.back() == ' ') s.pop_back();  // trim()
  if (s == "GENERAL") g_opttype = SDG_OPT_GENERAL;
  else if (s == "OPT1") g_opttype = SDG_OPT_OPT1;
  else if (s == "EVENODD") g_opttype = SDG_OPT_EVENODD;
  else return fail(SDG_ERR_BAD_OPTTYPE, "Unsupported dgoptr_evaltype: %s", t);
  return SDG_OK;
}

int sdg_dg_optr_kernel_type(void) { return g_opttype.load(); }

int sdg_evenodd_tables(int Nq, const double* D1D, const double* Lift_mat, double* tables) {
  if (!D1D || !Lift_mat || !tables) return fail(SDG_ERR_INVALID_ARG, "NULL argument");
  if (Nq - 1 < 1 || Nq - 1 > kMaxOrder)
    return fail(SDG_ERR_UNSUPPORTED_ORDER, "PolyOrder %d outside 1..15", Nq - 1);
  std::vector<double> tab;
  SDG_TRY(eo_tables(Nq, D1D, Lift_mat, tab));
  std::copy(tab.begin(), tab.end(), tables);
  return SDG_OK;
}

}  // extern "C"
