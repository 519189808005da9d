// Batched advance of many independent boxes (an ensemble, or the requests a
// server holds) with one launch per order present and RK stage.
//
// Every box is an instance with its own order p, size, dt, rotating state
// buffers and velocity.  A work item is one block's worth of consecutive
// elements of one instance.  The item list is sorted by order; each order's
// items run in one launch of a kernel compiled for that order and body:
// one block per item for the even-odd body (batch_one_item), or persistent
// blocks that take items round-robin and prefetch the next item's instance
// header into shared memory while computing the current one.  A block
// resolves the instance's buffers for the stage and runs the same fused
// stage body as the single-box solver (stage_block or stage_eo_block, FP32
// compute, FP64 state).  Each instance's current
// buffer index lives on the device and is advanced by a tiny kernel after
// stage 3, so one captured CUDA graph replays every step.
#pragma once

#include <vector>

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
  int body;  // 2 p + eo of the instance when the items were built: the stage
             // body the single-launch kernel runs (the groups use the same)
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

// The items of one order and stage body, run by one launch of a kernel
// compiled for that order and body.  The item list is sorted by order
// (and body), so a group is a contiguous range of it.
struct BatchGroup {
  int p = 0, eo = 0;       // order, 1 for the even-odd body
  int begin = 0, count = 0;  // item range
  int threads = 256;       // block size
  size_t smem = 0;         // dynamic shared memory of a block
  int grid = 0;            // blocks: one per item (one-item kernel) or the
                           // resident blocks, at most count (persistent kernel)
};

// Default block size and elements per work item of order p (1..11): the
// autotuner's choices for the even-odd body on four boxes of about 3.5M DOF
// of each order, on GB300.
void batch_default_shape(int p, int* threads, int* epb);
// Default stage body of order p (1: even-odd, 0: node body): the faster one
// in the batched kernels on GB300, which is the even-odd body at every order
// (at p = 2 since its lines take one thread each: 59.7 against 53.3
// GDOF-updates/s for the node body).
int batch_default_eo(int p);

// Sets the group kernel's shared-memory limit and its grid from occupancy.
int batch_group_setup(BatchGroup& g);
// Launches stage `stage` (0..2) of one group.
int batch_group_launch(const BatchInst* d_inst, const BatchItem* d_items, const BatchGroup& g,
                       int stage, cudaStream_t st);
// Splits a sorted item list into groups (epb and block size by order) and
// sets each up.
int batch_groups(const std::vector<BatchItem>& items, const std::vector<BatchInst>& inst,
                 const int* epb, const int* threads, std::vector<BatchGroup>& groups);
// cur = (cur + 1) % 3 for every active instance.
int batch_advance_launch(BatchInst* d_inst, int n_inst, cudaStream_t st);

// One side stream per order group, when `parallel` is set.  Groups touch
// disjoint instances, so a step can fork from the caller's stream into the
// groups' streams (each runs its group's three stages in order) and join
// them before the index advance, letting a small group's blocks fill the
// tail of a large group's launch.  Measured on GB300 it is slower (333
// against 369 solves/s on a 256-member ensemble of orders 3, 5 and 7; 27.4
// against 28.8 on the saturated serving stream), so the default runs the
// groups one after the other on the caller's stream.
struct BatchForkJoin {
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> done;
  cudaEvent_t fork = nullptr;
  bool parallel = false;  // false: every group on the caller's stream
  // true: each stage is ONE persistent launch over the items of every order
  // (batch_stage_kernel), instead of one launch per order group
  bool fused = false;
  BatchForkJoin() = default;
  BatchForkJoin(const BatchForkJoin&) = delete;
  BatchForkJoin& operator=(const BatchForkJoin&) = delete;
  ~BatchForkJoin();
};
// Enqueues one step of all groups on `st` (forked over the groups when
// there are several) and the index advance of n_inst instances.  Works
// under stream capture.
int batch_step_enqueue(BatchForkJoin& fj, BatchInst* d_inst, int n_inst,
                       const BatchItem* d_items, const std::vector<BatchGroup>& groups,
                       cudaStream_t st);
// Dynamic shared memory the kernel needs for `epb` elements of order p with
// the node body (eo = 0) or the even-odd body (eo = 1).
size_t batch_smem_bytes(int p, int epb, int eo);

// Device-side initial condition: Gaussian tracer exp(-d^2/(2 sigma^2)) around
// `centre` (periodic minimum image on the unit box) and a constant velocity,
// written into an instance's current state buffer and velocity arrays.
int batch_init_blob(const BatchInst& inst, const double* d_x1D, const double centre[3],
                    double sigma, const double vel[3], cudaStream_t st);

}  // namespace sdg
