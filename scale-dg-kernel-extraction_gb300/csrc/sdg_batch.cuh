// Batched advance of many independent boxes (an ensemble, or the requests a
// server holds) in ONE persistent launch per RK stage.
//
// Every box is an instance with its own order p, size, dt, rotating state
// buffers and velocity.  A work item is one block's worth of consecutive
// elements of one instance.  The persistent kernel's blocks take items
// round-robin from the list (sorted by order), prefetch the next item's
// instance header into shared memory while computing the current one, resolve
// the instance's buffers for the stage, and run the same fused stage body as
// the single-box solver (stage_block or stage_eo_block, FP32 compute, FP64
// state), dispatched on the instance's order.  Each instance's current
// buffer index lives on the device and is advanced by a tiny kernel after
// stage 3, so one captured CUDA graph replays every step.
#pragma once

#include "sdg_stage_eo.cuh"

namespace sdg {

constexpr int kBatchMaxOrder = 11;  // orders the batched kernel compiles
constexpr int kBatchThreadsMax = 512;

struct BatchInst {
  double* q[3];        // rotating FP64 state buffers
  const float* u;      // FP32 velocity
  const float* v;
  const float* w;
  const float* D;      // FP32 D1D(Nq,Nq) of this order
  const float* Lift;   // FP32 Lift_mat of this order
  const float* eo_tab; // FP32 even-odd tables of this order (or null)
  Box box;
  double dt;
  float cdt[3];        // FP32 b_s*dt of the three stages, made on the host
  float eo_sD[3][3];   // even-odd table factors per stage and direction:
  float eo_sL[3][3];   // -b_s*dt*Es_d and -b_s*dt*Fs_d/4
  int p;
  int eo;              // 1: the even-odd body, 0: the node body
  int cur;             // buffer holding the current state
  int active;          // 0: skipped by the stage kernel and by the advance
};

struct BatchItem {
  int inst;
  int e_begin;
  int e_count;
};

// FP32 increment factors b_s*dt of the three SSP-RK3 stages (mod_common.f90:30).
inline void batch_stage_factors(BatchInst& I) {
  const double b[3] = {1.0, 0.25, 2.0 / 3.0};
  for (int s = 0; s < 3; s++) {
    I.cdt[s] = (float)(b[s] * I.dt);
    const double c = b[s] * I.dt;
    for (int d = 0; d < 3; d++) {
      I.eo_sD[s][d] = (float)(-c * I.box.Es[d]);
      I.eo_sL[s][d] = (float)(-c * (0.25 * I.box.Fs[d]));
    }
  }
}

// Launches one stage over `n_items` items.
// mode: 0 all instances run the node body, 1 all the even-odd body, 2 mixed
// (batch_mode below).
int batch_stage_launch(const BatchInst* d_inst, const BatchItem* d_items, int n_items, int stage,
                       int grid, int threads, size_t smem, int mode, cudaStream_t st);
template <typename It, typename Get>
inline int batch_mode(It begin, It end, Get eo_of) {
  bool any_eo = false, any_node = false;
  for (It i = begin; i != end; ++i) (eo_of(*i) ? any_eo : any_node) = true;
  return any_eo ? (any_node ? 2 : 1) : 0;
}
// cur = (cur + 1) % 3 for every active instance.
int batch_advance_launch(BatchInst* d_inst, int n_inst, cudaStream_t st);
// Dynamic shared memory the kernel needs for `epb` elements of order p with
// the node body (eo = 0) or the even-odd body (eo = 1).
size_t batch_smem_bytes(int p, int epb, int eo);
// Resident blocks of the batch kernel per SM for a block size and smem size.
int batch_blocks_per_sm(int threads, size_t smem, int mode);
int batch_set_max_smem(size_t smem, int mode);

// Device-side initial condition: Gaussian tracer exp(-d^2/(2 sigma^2)) around
// `centre` (periodic minimum image on the unit box) and a constant velocity,
// written into an instance's current state buffer and velocity arrays.
int batch_init_blob(const BatchInst& inst, const double* d_x1D, const double centre[3],
                    double sigma, const double vel[3], cudaStream_t st);

}  // namespace sdg
