// Device-side construction of the reference's mesh arrays (mesh_setup,
// mod_mesh.f90:74-193, with element_init's face tables :265-324,
// set_element_position :332-353, set_face_geometry :356-397 and
// eval_neighbor_element :407-483) for the periodic box.
//
// The arrays are those the drop-in sdg_advect3d_eq_cal_tend_dev consumes:
// VMapM / VMapP (1-based; periodic faces point into the halo buffer),
// normal_fn, Escale, Fscale, pos_en and halo_src_map.  The only serial part of
// mesh_setup is the halo-slot numbering (mod_mesh.f90:171-190: a running
// counter over elements in k, j, i order, faces 1..6, face nodes); its
// per-element starting offsets are an O(Ne) prefix computed on the host, and
// every per-node and per-face-node value is computed on the device in
// parallel.  Floating-point values use the reference's formulas with
// separately rounded operations (no contraction into FMA), so they equal the
// host-built arrays bit for bit.
#include <cuda_runtime.h>

#include <vector>

#include "sdg_internal.h"

using namespace sdg;

namespace {

struct MeshArgs {
  int NeX, NeY, NeZ, Nq, Np, Nfp, NfpTot;
  long long Ne;
  double dx, dy, dz;
  const double* x1D;       // device, Nq
  const int* halo_off;     // device, Ne: first halo slot (0-based) of each element
  int* VMapM;
  int* VMapP;
  double* normal_fn;
  double* Escale;
  double* Fscale;
  double* pos_en;
  int* halo_src_map;
};

// Fmask(fp, f) (1-based node id), mod_mesh.f90:278-324, for tangential
// indices (a, b) of face node fp = a + b*Nq.
__device__ int fmask(int f, int a, int b, int Nq) {
  const int Q2 = Nq * Nq;
  switch (f) {
    case 1: return 1 + a + b * Q2;                    // (i, k): i + (k-1) Nq^2
    case 2: return Nq + a * Nq + b * Q2;              // (j, k)
    case 3: return 1 + a + (Nq - 1) * Nq + b * Q2;    // (i, k)
    case 4: return 1 + a * Nq + b * Q2;               // (j, k)
    case 5: return 1 + a + b * Nq;                    // (i, j)
    default: return 1 + a + b * Nq + (Nq - 1) * Q2;  // (i, j)
  }
}

__global__ void face_kernel(const MeshArgs m) {
  const long long NT = (long long)m.NfpTot * m.Ne;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < NT;
       t += (long long)gridDim.x * blockDim.x) {
    const long long e0 = t / m.NfpTot;
    const int r = (int)(t - e0 * m.NfpTot);
    const int f = r / m.Nfp + 1;  // 1-based face
    const int fp = r % m.Nfp;
    const int a = fp % m.Nq, b = fp / m.Nq;
    const int ei = (int)(e0 % m.NeX) + 1;
    const int ej = (int)((e0 / m.NeX) % m.NeY) + 1;
    const int ek = (int)(e0 / ((long long)m.NeX * m.NeY)) + 1;
    int ni = ei, nj = ej, nk = ek, opp = 0;
    bool bnd = false;
    switch (f) {
      case 1: opp = 3; bnd = (ej == 1); nj = bnd ? m.NeY : ej - 1; break;
      case 2: opp = 4; bnd = (ei == m.NeX); ni = bnd ? 1 : ei + 1; break;
      case 3: opp = 1; bnd = (ej == m.NeY); nj = bnd ? 1 : ej + 1; break;
      case 4: opp = 2; bnd = (ei == 1); ni = bnd ? m.NeX : ei - 1; break;
      case 5: opp = 6; bnd = (ek == 1); nk = bnd ? m.NeZ : ek - 1; break;
      default: opp = 5; bnd = (ek == m.NeZ); nk = bnd ? 1 : ek + 1; break;
    }
    const long long keP = ni + (long long)(nj - 1) * m.NeX + (long long)(nk - 1) * m.NeX * m.NeY;
    const int src = fmask(opp, a, b, m.Nq) + (int)((keP - 1) * m.Np);
    if (m.VMapM) m.VMapM[t] = fmask(f, a, b, m.Nq) + (int)(e0 * m.Np);
    if (bnd) {
      // boundary faces of this element before face f, in face order
      const bool fb[7] = {false, ej == 1, ei == m.NeX, ej == m.NeY, ei == 1, ek == 1, ek == m.NeZ};
      int before = 0;
      for (int g = 1; g < f; g++) before += fb[g] ? 1 : 0;
      const long long slot = (long long)m.halo_off[e0] + (long long)before * m.Nfp + fp;
      if (m.VMapP) m.VMapP[t] = (int)((long long)m.Np * m.Ne + slot + 1);
      if (m.halo_src_map) m.halo_src_map[slot] = src;
    } else if (m.VMapP) {
      m.VMapP[t] = src;
    }
    // set_face_geometry: axis-aligned unit normals and Fscale = 2/h
    const int axis = (f == 2 || f == 4) ? 0 : (f == 1 || f == 3) ? 1 : 2;
    const double sgn = (f == 2 || f == 3 || f == 6) ? 1.0 : -1.0;
    if (m.normal_fn)
      for (int d = 0; d < 3; d++) m.normal_fn[t + d * NT] = (d == axis) ? sgn : 0.0;
    if (m.Fscale) {
      const double h = (axis == 0) ? m.dx : (axis == 1) ? m.dy : m.dz;
      m.Fscale[t] = __ddiv_rn(2.0, h);
    }
  }
}

__global__ void node_kernel(const MeshArgs m) {
  const long long N = (long long)m.Np * m.Ne;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < N;
       t += (long long)gridDim.x * blockDim.x) {
    const long long e0 = t / m.Np;
    const int n = (int)(t - e0 * m.Np);
    const int i = n % m.Nq, j = (n / m.Nq) % m.Nq, k = n / (m.Nq * m.Nq);
    const int ei = (int)(e0 % m.NeX) + 1;
    const int ej = (int)((e0 / m.NeX) % m.NeY) + 1;
    const int ek = (int)(e0 / ((long long)m.NeX * m.NeY)) + 1;
    if (m.Escale) {
      m.Escale[t] = __ddiv_rn(2.0, m.dx);
      m.Escale[t + N] = __ddiv_rn(2.0, m.dy);
      m.Escale[t + 2 * N] = __ddiv_rn(2.0, m.dz);
    }
    if (m.pos_en) {
      // xc + (0.5*dx)*x1D(i) with xc = (real(i) - 0.5)*dx, each operation rounded
      const double xc = __dmul_rn(__dadd_rn((double)ei, -0.5), m.dx);
      const double yc = __dmul_rn(__dadd_rn((double)ej, -0.5), m.dy);
      const double zc = __dmul_rn(__dadd_rn((double)ek, -0.5), m.dz);
      m.pos_en[t] = __dadd_rn(xc, __dmul_rn(__dmul_rn(0.5, m.dx), m.x1D[i]));
      m.pos_en[t + N] = __dadd_rn(yc, __dmul_rn(__dmul_rn(0.5, m.dy), m.x1D[j]));
      m.pos_en[t + 2 * N] = __dadd_rn(zc, __dmul_rn(__dmul_rn(0.5, m.dz), m.x1D[k]));
    }
  }
}

unsigned grid_for(long long n) {
  long long nb = (n + 255) / 256;
  if (nb > 152LL * 64) nb = 152LL * 64;
  return (unsigned)(nb > 0 ? nb : 1);
}

}  // namespace

extern "C" int sdg_mesh_setup_dev(int NeX, int NeY, int NeZ, int p, double Lx, double Ly,
                                  double Lz, const double* x1D, int* VMapM, int* VMapP,
                                  double* normal_fn, double* Escale, double* Fscale,
                                  double* pos_en, int* halo_src_map, void* stream) {
  if (p < 1 || p > kMaxOrder)
    return fail(SDG_ERR_UNSUPPORTED_ORDER, "PolyOrder %d outside 1..15", p);
  if (NeX < 1 || NeY < 1 || NeZ < 1 || !(Lx > 0) || !(Ly > 0) || !(Lz > 0))
    return fail(SDG_ERR_INVALID_ARG, "bad box");
  const int Nq = p + 1, Np = Nq * Nq * Nq, Nfp = Nq * Nq, NfpTot = 6 * Nfp;
  const long long Ne = (long long)NeX * NeY * NeZ;
  const long long nhalo = 2LL * ((long long)NeY * NeZ + (long long)NeX * NeZ + (long long)NeX * NeY);
  if ((long long)Np * (Ne + nhalo) > 0x7fffffffLL)
    return fail(SDG_ERR_INVALID_ARG, "mesh too large for 32-bit VMap indices");
  if (!x1D && pos_en) return fail(SDG_ERR_INVALID_ARG, "pos_en needs x1D");
  SDG_TRY(require_device());
  // halo-slot offsets in the serial order of mod_mesh.f90:171-190
  std::vector<int> off((size_t)Ne);
  long long acc = 0;
  for (int k = 1; k <= NeZ; k++)
    for (int j = 1; j <= NeY; j++)
      for (int i = 1; i <= NeX; i++) {
        off[(size_t)(i - 1 + (long long)(j - 1) * NeX + (long long)(k - 1) * NeX * NeY)] = (int)acc;
        const int nb = (j == 1) + (i == NeX) + (j == NeY) + (i == 1) + (k == 1) + (k == NeZ);
        acc += (long long)nb * Nfp;
      }
  cudaStream_t st = as_stream(stream);
  int* d_off = nullptr;
  double* d_x = nullptr;
  SDG_CUDA_TRY(cudaMalloc(&d_off, sizeof(int) * (size_t)Ne));
  cudaError_t e = cudaMalloc(&d_x, sizeof(double) * Nq);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_off, off.data(), sizeof(int) * (size_t)Ne, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && x1D)
    e = cudaMemcpyAsync(d_x, x1D, sizeof(double) * Nq, cudaMemcpyHostToDevice, st);
  MeshArgs m{NeX, NeY, NeZ, Nq, Np, Nfp, NfpTot, Ne, Lx / (double)NeX, Ly / (double)NeY,
             Lz / (double)NeZ, d_x, d_off, VMapM, VMapP, normal_fn, Escale, Fscale, pos_en,
             halo_src_map};
  if (e == cudaSuccess) {
    face_kernel<<<grid_for((long long)NfpTot * Ne), 256, 0, st>>>(m);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    node_kernel<<<grid_for((long long)Np * Ne), 256, 0, st>>>(m);
    e = cudaGetLastError();
  }
  // the host offsets must outlive the copy; the temporaries are freed after it
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d_off);
  cudaFree(d_x);
  if (e != cudaSuccess) return cuda_fail(e, "device mesh setup", __FILE__, __LINE__);
  return SDG_OK;
}
