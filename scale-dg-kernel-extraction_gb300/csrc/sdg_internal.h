// Internal declarations shared by the translation units of libsdg_gb300.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <vector>

#include "sdg_advect.h"

namespace sdg {

constexpr int kMaxOrder = 15;

// Records a message for sdg_last_error() (thread-local) and returns status.
int fail(int status, const char* fmt, ...);
// Maps a CUDA error to SDG_ERR_CUDA / SDG_ERR_OUT_OF_MEMORY with a message.
int cuda_fail(cudaError_t e, const char* what, const char* file, int line);

#define SDG_CUDA_TRY(call)                                              \
  do {                                                                  \
    cudaError_t sdg_e_ = (call);                                        \
    if (sdg_e_ != cudaSuccess)                                          \
      return ::sdg::cuda_fail(sdg_e_, #call, __FILE__, __LINE__);       \
  } while (0)

#define SDG_TRY(expr)                 \
  do {                                \
    int sdg_s_ = (expr);              \
    if (sdg_s_ != SDG_OK) return sdg_s_; \
  } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Raises a kernel's dynamic shared-memory limit to smem bytes (and, when
// asked, prefers the largest shared-memory carveout) on the current device.
// Kernel attributes are per device, so this records (kernel, device, smem)
// and sets them once per device; it is safe to call from several host
// threads at once.
int set_kernel_smem(const void* func, int smem, bool max_carveout);

// Checks the first CUDA device is usable; returns SDG_OK or an error status.
int require_device();

// Structured periodic box: what the fused stage kernel needs to know about the
// mesh of mod_mesh.f90:74-193 (element order, per-axis scale factors).
struct Box {
  int NeX, NeY, NeZ;
  long long Ne;
  double Es[3];  // Escale(:,:,d) = 2/dx_d  (mod_mesh.f90:147-149)
  double Fs[3];  // Fscale of the faces normal to axis d (mod_mesh.f90:366-394)
  // FP32 copies made on the host (Es, and 0.5*Fs as the flux uses it): a
  // conversion in the kernel would run on GB300's 1/64-rate FP64 pipe
  float Esf[3];
  float hFsf[3];
};
Box make_box(int NeX, int NeY, int NeZ, double Lx, double Ly, double Lz);

// Arguments of one fused stage launch.
struct StageArgs {
  const double* q_in;   // state read by the stage (Np*Ne)
  const double* q0;     // step-start state (stages 2 and 3), may be null if a==0
  double* q_out;        // RK result (Np*Ne), or the tendency when tend_only
  const void* u;        // velocity components (double or float, Np*Ne)
  const void* v;
  const void* w;
  const void* D;        // D1D(Nq,Nq), column-major, compute type
  const void* Lift;     // Lift_mat(Nq,Nq,Nq,6), compute type
  Box box;
  long long elem_begin;  // first element of this launch
  long long elem_count;  // elements of this launch
  double a, b, dt;      // q_out = a*q0 + b*(q_in + dt*dqdt)
  float cdt_hi, cdt_lo; // b*dt as a double-float pair (emulated-FP64 kernel)
  int b_is_one;         // b == 1 (stage 1): the kernels branch on integers,
  int a_nonzero;        // since an FP64 comparison also uses the FP64 pipe
  int tend_only;        // write dqdt instead of the RK update
  // even-odd FP64 stage: per-direction factors of the D part (-c*Es_d) and
  // of the lift part (-c*Fs_d/4) of the tables, c = b*dt (1 for tend_only);
  // D then points at the 3-direction table built by the solver
  double eo_sD[3], eo_sL[3];
  float eo_sDf[3], eo_sLf[3];  // the same factors for the FP32-compute form
  // even-odd FP64 stage: the velocity factors of the face flux, (tP, tM) per
  // face node of each element (2*Nfp*6 doubles an element).  A stage with
  // fc_out forms them from u, v, w and stores them; a stage with fc_in reads
  // them instead (same bits), so the stages of one solver call, which share
  // the velocity (main.f90:58-67 passes the same u, v, w to every
  // advect3d_eq_cal_tend call), form them once.  Both null: formed inline.
  double* fc_out;
  const double* fc_in;
};

// Even-odd tables (3 directions, unscaled) from D1D and Lift_mat after the
// symmetry checks; SDG_ERR_INVALID_ARG when the operators lack them.
int eo_tables(int Nq, const double* D1D, const double* Lift_mat, std::vector<double>& tab);

// Fused stage launchers (sdg_stage_*.cu).  prec = SDG_PREC_*.
int launch_stage(int p, int prec, int opt, const StageArgs& a, cudaStream_t st);

// min / max of q[0..n) as order keys (see sdg_minmax.cu); resets both keys first.
int minmax_launch(const double* q, long long n, unsigned long long* kmin, unsigned long long* kmax,
                  cudaStream_t st);
double minmax_key_to_double(unsigned long long k);
// Dynamic shared memory the launcher uses for order p, to size opt-in limits.
int stage_setup_attributes(int p, int prec, int opt);

}  // namespace sdg
