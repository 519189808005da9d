// Ensemble of independent boxes advanced together (sdg_ensemble_* in
// include/sdg_advect.h): all instances live in one device arena; a step is a
// CUDA graph of [3 persistent stage launches, advance].
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <new>
#include <vector>

#include "sdg_batch.cuh"
#include "sdg_internal.h"

using namespace sdg;

struct sdg_ensemble {
  int n = 0;
  std::vector<BatchInst> inst;     // host mirror (buffer pointers, sizes)
  std::vector<int> cur_host;       // current buffer index per instance
  BatchInst* d_inst = nullptr;
  BatchItem* d_items = nullptr;
  int n_items = 0;
  void* arena = nullptr;
  float* d_ops[kBatchMaxOrder + 1][3] = {};  // D1D, Lift, even-odd tables (FP32)
  int eo_by_order[kBatchMaxOrder + 1] = {};  // stage body per order (1: even-odd)
  bool body_fixed = false;         // set_opt chose the body; the tuner keeps it
  double* d_x1D[kBatchMaxOrder + 1] = {};
  int epb[kBatchMaxOrder + 1] = {};
  int threads[kBatchMaxOrder + 1] = {};
  std::vector<BatchGroup> groups;  // one persistent launch per order present
  BatchForkJoin fj;                // a side stream per group
  cudaStream_t stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  long long total_dof = 0;
};

namespace {

void free_ensemble(sdg_ensemble* e) {
  if (e->graph) cudaGraphExecDestroy(e->graph);
  cudaFree(e->d_inst);
  cudaFree(e->d_items);
  cudaFree(e->arena);
  for (int p = 0; p <= kBatchMaxOrder; p++) {
    cudaFree(e->d_ops[p][0]);
    cudaFree(e->d_ops[p][1]);
    cudaFree(e->d_ops[p][2]);
    cudaFree(e->d_x1D[p]);
  }
}

// Work items for the current elements-per-block choice, most expensive
// orders first so that the tail of the persistent loop holds cheap items.
int build_items(sdg_ensemble* e, const std::vector<int>* subset = nullptr) {
  std::vector<BatchItem> items;
  std::vector<int> idx;
  if (subset) idx = *subset;
  else
    for (int i = 0; i < e->n; i++) idx.push_back(i);
  std::stable_sort(idx.begin(), idx.end(),
                   [&](int a, int b) { return e->inst[a].p > e->inst[b].p; });
  for (int i : idx) {
    const BatchInst& I = e->inst[i];
    const int epb = e->epb[I.p];
    for (long long b = 0; b < I.box.Ne; b += epb)
      items.push_back({i, (int)b, (int)std::min<long long>(epb, I.box.Ne - b),
                       2 * I.p + (I.eo ? 1 : 0)});
  }
  cudaFree(e->d_items);
  e->d_items = nullptr;
  e->n_items = (int)items.size();
  if (!items.empty()) {
    SDG_CUDA_TRY(cudaMalloc(&e->d_items, sizeof(BatchItem) * items.size()));
    SDG_CUDA_TRY(cudaMemcpy(e->d_items, items.data(), sizeof(BatchItem) * items.size(),
                            cudaMemcpyHostToDevice));
  }
  return batch_groups(items, e->inst, e->epb, e->threads, e->groups);
}

int enqueue_step(sdg_ensemble* e) {
  return batch_step_enqueue(e->fj, e->d_inst, e->n, e->d_items, e->groups, e->stream);
}

int capture_graph(sdg_ensemble* e) {
  if (e->graph) {
    cudaGraphExecDestroy(e->graph);
    e->graph = nullptr;
  }
  cudaStream_t cs;
  SDG_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  cudaStream_t saved = e->stream;
  e->stream = cs;
  cudaGraph_t g = nullptr;
  cudaError_t ce = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  int st = SDG_OK;
  if (ce == cudaSuccess) st = enqueue_step(e);
  cudaError_t ce2 = cudaStreamEndCapture(cs, &g);
  e->stream = saved;
  cudaStreamDestroy(cs);
  if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamBeginCapture", __FILE__, __LINE__);
  if (st != SDG_OK) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  if (ce2 != cudaSuccess) return cuda_fail(ce2, "cudaStreamEndCapture", __FILE__, __LINE__);
  ce = cudaGraphInstantiate(&e->graph, g, 0);
  cudaGraphDestroy(g);
  if (ce != cudaSuccess) return cuda_fail(ce, "cudaGraphInstantiate", __FILE__, __LINE__);
  return SDG_OK;
}

int time_stage0(sdg_ensemble* e, float* ms) {
  cudaEvent_t a, b;
  SDG_CUDA_TRY(cudaEventCreate(&a));
  SDG_CUDA_TRY(cudaEventCreate(&b));
  float best = 1e30f;
  for (int r = 0; r < 3; r++) {
    // stage 0 reads q[cur] and writes q[cur+1]: repeating it leaves the state
    SDG_CUDA_TRY(cudaEventRecord(a, e->stream));
    for (const BatchGroup& g : e->groups)
      SDG_TRY(batch_group_launch(e->d_inst, e->d_items, g, 0, e->stream));
    SDG_CUDA_TRY(cudaEventRecord(b, e->stream));
    SDG_CUDA_TRY(cudaEventSynchronize(b));
    float t = 0.f;
    SDG_CUDA_TRY(cudaEventElapsedTime(&t, a, b));
    best = std::min(best, t);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *ms = best;
  return SDG_OK;
}

}  // namespace

extern "C" {

int sdg_ensemble_create(sdg_ensemble** out, int n, const int* dims, const int* orders,
                        const double* dt, const double* const* D1D_by_order,
                        const double* const* Lift_by_order, const double* const* x1D_by_order,
                        void* stream) {
  if (!out) return fail(SDG_ERR_INVALID_ARG, "NULL output handle");
  *out = nullptr;
  if (n < 1 || !dims || !orders || !dt || !D1D_by_order || !Lift_by_order)
    return fail(SDG_ERR_INVALID_ARG, "bad ensemble description");
  for (int i = 0; i < n; i++) {
    if (orders[i] < 1 || orders[i] > kBatchMaxOrder)
      return fail(SDG_ERR_UNSUPPORTED_ORDER, "instance %d: order %d outside 1..%d", i,
                  orders[i], kBatchMaxOrder);
    if (dims[3 * i] < 1 || dims[3 * i + 1] < 1 || dims[3 * i + 2] < 1 || !(dt[i] > 0))
      return fail(SDG_ERR_INVALID_ARG, "instance %d: bad size or dt", i);
    if (!D1D_by_order[orders[i]] || !Lift_by_order[orders[i]])
      return fail(SDG_ERR_INVALID_ARG, "no operators for order %d", orders[i]);
  }
  SDG_TRY(require_device());
  sdg_ensemble* e = new (std::nothrow) sdg_ensemble();
  if (!e) return fail(SDG_ERR_OUT_OF_MEMORY, "host allocation failed");
  e->n = n;
  e->stream = as_stream(stream);
  e->inst.resize(n);
  e->cur_host.assign(n, 0);
  for (int p = 0; p <= kBatchMaxOrder; p++) batch_default_shape(p, &e->threads[p], &e->epb[p]);
  auto bail = [&](int st) {
    free_ensemble(e);
    delete e;
    return st;
  };
  // operators per order, in FP32 (and x1D in FP64 for the device initial condition)
  for (int i = 0; i < n; i++) {
    const int p = orders[i];
    if (e->d_ops[p][0]) continue;
    const int nq = p + 1, nd = nq * nq, nl = 6 * nq * nq * nq;
    std::vector<float> d(nd), l(nl);
    for (int k = 0; k < nd; k++) d[k] = (float)D1D_by_order[p][k];
    for (int k = 0; k < nl; k++) l[k] = (float)Lift_by_order[p][k];
    cudaError_t ce = cudaMalloc(&e->d_ops[p][0], 4 * nd);
    if (ce == cudaSuccess) ce = cudaMalloc(&e->d_ops[p][1], 4 * nl);
    if (ce == cudaSuccess) ce = cudaMemcpy(e->d_ops[p][0], d.data(), 4 * nd, cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(e->d_ops[p][1], l.data(), 4 * nl, cudaMemcpyHostToDevice);
    if (ce == cudaSuccess && x1D_by_order && x1D_by_order[p]) {
      ce = cudaMalloc(&e->d_x1D[p], 8 * nq);
      if (ce == cudaSuccess) ce = cudaMemcpy(e->d_x1D[p], x1D_by_order[p], 8 * nq, cudaMemcpyHostToDevice);
    }
    // even-odd tables when the operators have the centro-symmetry
    std::vector<double> eo;
    if (ce == cudaSuccess && eo_tables(nq, D1D_by_order[p], Lift_by_order[p], eo) == SDG_OK) {
      std::vector<float> ef(eo.begin(), eo.end());
      ce = cudaMalloc(&e->d_ops[p][2], 4 * ef.size());
      if (ce == cudaSuccess)
        ce = cudaMemcpy(e->d_ops[p][2], ef.data(), 4 * ef.size(), cudaMemcpyHostToDevice);
    }
    if (ce != cudaSuccess) return bail(cuda_fail(ce, "ensemble operators", __FILE__, __LINE__));
  }
  // one arena: per instance 3 FP64 state buffers and 3 FP32 velocity arrays
  size_t bytes = 0;
  std::vector<size_t> off(n);
  for (int i = 0; i < n; i++) {
    const long long np = (long long)(orders[i] + 1) * (orders[i] + 1) * (orders[i] + 1);
    const long long nd = np * dims[3 * i] * dims[3 * i + 1] * dims[3 * i + 2];
    off[i] = bytes;
    bytes += ((size_t)nd * (3 * 8 + 3 * 4) + 255) & ~(size_t)255;
    e->total_dof += nd;
  }
  cudaError_t ce = cudaMalloc(&e->arena, bytes);
  if (ce != cudaSuccess) return bail(cuda_fail(ce, "ensemble arena", __FILE__, __LINE__));
  for (int i = 0; i < n; i++) {
    BatchInst& I = e->inst[i];
    const int p = orders[i];
    const long long np = (long long)(p + 1) * (p + 1) * (p + 1);
    I.box = make_box(dims[3 * i], dims[3 * i + 1], dims[3 * i + 2], 1.0, 1.0, 1.0);
    const long long nd = np * I.box.Ne;
    char* base = static_cast<char*>(e->arena) + off[i];
    for (int k = 0; k < 3; k++) I.q[k] = reinterpret_cast<double*>(base + 8 * nd * k);
    float* vel = reinterpret_cast<float*>(base + 24 * nd);
    I.u = vel;
    I.v = vel + nd;
    I.w = vel + 2 * nd;
    I.D = e->d_ops[p][0];
    I.Lift = e->d_ops[p][1];
    I.eo_tab = e->d_ops[p][2];
    e->eo_by_order[p] = (I.eo_tab != nullptr) ? 1 : 0;  // even-odd by default
    I.eo = e->eo_by_order[p];
    I.dt = dt[i];
    batch_stage_factors(I);
    I.p = p;
    I.cur = 0;
    I.active = 1;
  }
  ce = cudaMalloc(&e->d_inst, sizeof(BatchInst) * n);
  if (ce == cudaSuccess)
    ce = cudaMemcpy(e->d_inst, e->inst.data(), sizeof(BatchInst) * n, cudaMemcpyHostToDevice);
  if (ce != cudaSuccess) return bail(cuda_fail(ce, "ensemble tables", __FILE__, __LINE__));
  int st = build_items(e);
  if (st != SDG_OK) return bail(st);
  *out = e;
  return SDG_OK;
}

int sdg_ensemble_upload(sdg_ensemble* e, int i, const double* q, const double* u,
                        const double* v, const double* w) {
  if (!e || i < 0 || i >= e->n || !q || !u || !v || !w)
    return fail(SDG_ERR_INVALID_ARG, "bad ensemble upload");
  const BatchInst& I = e->inst[i];
  const long long nd = (long long)(I.p + 1) * (I.p + 1) * (I.p + 1) * I.box.Ne;
  SDG_CUDA_TRY(cudaMemcpy(I.q[e->cur_host[i]], q, 8 * nd, cudaMemcpyHostToDevice));
  std::vector<float> f(nd);
  const double* src[3] = {u, v, w};
  const float* dst[3] = {I.u, I.v, I.w};
  for (int c = 0; c < 3; c++) {
    for (long long k = 0; k < nd; k++) f[k] = (float)src[c][k];
    SDG_CUDA_TRY(cudaMemcpy(const_cast<float*>(dst[c]), f.data(), 4 * nd, cudaMemcpyHostToDevice));
  }
  return SDG_OK;
}

int sdg_ensemble_init_blob(sdg_ensemble* e, int i, const double* centre, double sigma,
                           const double* velocity) {
  if (!e || i < 0 || i >= e->n || !centre || !velocity || !(sigma > 0))
    return fail(SDG_ERR_INVALID_ARG, "bad ensemble initial condition");
  BatchInst I = e->inst[i];
  if (!e->d_x1D[I.p]) return fail(SDG_ERR_INVALID_ARG, "no x1D given for order %d", I.p);
  I.cur = e->cur_host[i];
  return batch_init_blob(I, e->d_x1D[I.p], centre, sigma, velocity, e->stream);
}

int sdg_ensemble_set_epb(sdg_ensemble* e, int p, int epb) {
  if (!e || p < 1 || p > kBatchMaxOrder || epb < 1 || epb > 256)
    return fail(SDG_ERR_INVALID_ARG, "bad elements-per-block choice");
  e->epb[p] = epb;
  if (e->graph) {
    cudaGraphExecDestroy(e->graph);
    e->graph = nullptr;
  }
  return build_items(e);
}

int sdg_ensemble_set_threads(sdg_ensemble* e, int threads) {
  if (!e || threads < 32 || threads > kBatchThreadsMax || threads % 32)
    return fail(SDG_ERR_INVALID_ARG, "bad block size %d", threads);
  for (int p = 0; p <= kBatchMaxOrder; p++) e->threads[p] = threads;
  if (e->graph) {
    cudaGraphExecDestroy(e->graph);
    e->graph = nullptr;
  }
  return build_items(e);
}

int sdg_ensemble_set_order_threads(sdg_ensemble* e, int p, int threads) {
  if (!e || p < 1 || p > kBatchMaxOrder || threads < 32 || threads > kBatchThreadsMax ||
      threads % 32)
    return fail(SDG_ERR_INVALID_ARG, "bad block size %d for order %d", threads, p);
  e->threads[p] = threads;
  if (e->graph) {
    cudaGraphExecDestroy(e->graph);
    e->graph = nullptr;
  }
  return build_items(e);
}

// The kernels take the stage body from their group, so a body change only
// regroups the items (the device instance table keeps its buffer indices).
static void set_bodies(sdg_ensemble* e) {
  for (int i = 0; i < e->n; i++) {
    BatchInst& I = e->inst[i];
    I.eo = (I.eo_tab != nullptr && e->eo_by_order[I.p]) ? 1 : 0;
  }
}

int sdg_ensemble_set_opt(sdg_ensemble* e, int opt) {
  if (!e) return fail(SDG_ERR_INVALID_ARG, "NULL ensemble");
  if (opt != SDG_OPT_GENERAL && opt != SDG_OPT_OPT1 && opt != SDG_OPT_EVENODD)
    return fail(SDG_ERR_BAD_OPTTYPE, "unknown opt type %d", opt);
  for (int p = 0; p <= kBatchMaxOrder; p++) e->eo_by_order[p] = (opt == SDG_OPT_EVENODD);
  e->body_fixed = true;
  set_bodies(e);
  if (e->graph) {
    cudaGraphExecDestroy(e->graph);
    e->graph = nullptr;
  }
  return build_items(e);
}

int sdg_ensemble_set_parallel_groups(sdg_ensemble* e, int on) {
  if (!e) return fail(SDG_ERR_INVALID_ARG, "NULL ensemble");
  e->fj.parallel = (on != 0);
  if (e->graph) {
    cudaGraphExecDestroy(e->graph);
    e->graph = nullptr;
  }
  return SDG_OK;
}

int sdg_ensemble_set_single_launch(sdg_ensemble* e, int on) {
  if (!e) return fail(SDG_ERR_INVALID_ARG, "NULL ensemble");
  e->fj.fused = (on != 0);
  if (e->graph) {
    cudaGraphExecDestroy(e->graph);
    e->graph = nullptr;
  }
  return SDG_OK;
}

int sdg_ensemble_get_threads(const sdg_ensemble* e, int* threads_by_order) {
  if (!e || !threads_by_order) return fail(SDG_ERR_INVALID_ARG, "NULL argument");
  for (int p = 0; p <= kBatchMaxOrder; p++) threads_by_order[p] = e->threads[p];
  return SDG_OK;
}

int sdg_ensemble_get_bodies(const sdg_ensemble* e, int* eo_by_order) {
  if (!e || !eo_by_order) return fail(SDG_ERR_INVALID_ARG, "NULL argument");
  for (int p = 0; p <= kBatchMaxOrder; p++) {
    int any = 0;
    for (int i = 0; i < e->n && !any; i++) any = (e->inst[i].p == p) ? e->inst[i].eo : 0;
    eo_by_order[p] = any;
  }
  return SDG_OK;
}

int sdg_ensemble_get_config(const sdg_ensemble* e, int* epb_by_order, int* threads, int* grid) {
  if (!e) return fail(SDG_ERR_INVALID_ARG, "NULL ensemble");
  if (epb_by_order)
    for (int p = 0; p <= kBatchMaxOrder; p++) epb_by_order[p] = e->epb[p];
  if (threads) {
    // the block size the present orders share, or 0 when they differ
    *threads = -1;
    for (int i = 0; i < e->n; i++) {
      const int t = e->threads[e->inst[i].p];
      *threads = (*threads == -1 || *threads == t) ? t : 0;
    }
    if (*threads < 0) *threads = 0;
  }
  if (grid) {
    *grid = 0;
    for (const BatchGroup& g : e->groups) *grid = std::max(*grid, g.grid);
  }
  return SDG_OK;
}

// Autotuner: for each order present, time stage 0 over that order's
// instances for both stage bodies (even-odd where the operators allow it, and
// the node body; after set_opt only the body it chose), each block size in
// {128, 256, 512} and every elements-per-block candidate (about 64 to 4096
// nodes a block, shared memory under 96 KB), and keep the fastest
// (body, block size, elements per block) of each order.  Stage 0 leaves the
// state unchanged, so tuning can run at any point.
int sdg_ensemble_tune(sdg_ensemble* e) {
  if (!e) return fail(SDG_ERR_INVALID_ARG, "NULL ensemble");
  std::vector<std::vector<int>> by_order(kBatchMaxOrder + 1);
  for (int i = 0; i < e->n; i++) by_order[e->inst[i].p].push_back(i);
  const int thread_opts[3] = {128, 256, 512};
  for (int p = 1; p <= kBatchMaxOrder; p++) {
    if (by_order[p].empty()) continue;
    const int np = (p + 1) * (p + 1) * (p + 1);
    const bool has_eo = e->inst[by_order[p][0]].eo_tab != nullptr;
    const int body_hi = e->body_fixed ? e->eo_by_order[p] : (has_eo ? 1 : 0);
    const int body_lo = e->body_fixed ? e->eo_by_order[p] : 0;
    float best = 1e30f;
    int best_eo = e->eo_by_order[p], best_th = e->threads[p], best_epb = e->epb[p];
    for (int body = body_hi; body >= body_lo; body--) {
      e->eo_by_order[p] = body;
      set_bodies(e);
      for (int th : thread_opts) {
        e->threads[p] = th;
        for (int cand = 1; cand <= 256; cand *= 2) {
          if (cand * np > 4096 || (cand * np < 64 && cand * 2 * np <= 4096)) continue;
          if (batch_smem_bytes(p, cand, body) > 96 * 1024) continue;
          e->epb[p] = cand;
          if (build_items(e, &by_order[p]) != SDG_OK) continue;
          float ms = 0.f;
          SDG_TRY(time_stage0(e, &ms));
          if (ms < best) {
            best = ms;
            best_eo = body;
            best_th = th;
            best_epb = cand;
          }
        }
      }
    }
    e->eo_by_order[p] = best_eo;
    e->threads[p] = best_th;
    e->epb[p] = best_epb;
    set_bodies(e);
  }
  if (e->graph) {
    cudaGraphExecDestroy(e->graph);
    e->graph = nullptr;
  }
  return build_items(e);
}

int sdg_ensemble_step(sdg_ensemble* e, int nstep) {
  if (!e || nstep < 0) return fail(SDG_ERR_INVALID_ARG, "bad ensemble step");
  if (!e->graph) SDG_TRY(capture_graph(e));
  for (int s = 0; s < nstep; s++) SDG_CUDA_TRY(cudaGraphLaunch(e->graph, e->stream));
  for (int i = 0; i < e->n; i++) e->cur_host[i] = (e->cur_host[i] + nstep) % 3;
  return SDG_OK;
}

int sdg_ensemble_step_timed(sdg_ensemble* e, int nstep, double* ms) {
  if (!e || !ms) return fail(SDG_ERR_INVALID_ARG, "NULL argument");
  if (!e->graph) SDG_TRY(capture_graph(e));
  cudaEvent_t a, b;
  SDG_CUDA_TRY(cudaEventCreate(&a));
  SDG_CUDA_TRY(cudaEventCreate(&b));
  SDG_CUDA_TRY(cudaEventRecord(a, e->stream));
  const int st = sdg_ensemble_step(e, nstep);
  SDG_CUDA_TRY(cudaEventRecord(b, e->stream));
  SDG_CUDA_TRY(cudaEventSynchronize(b));
  float f = 0.f;
  SDG_CUDA_TRY(cudaEventElapsedTime(&f, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *ms = f;
  return st;
}

int sdg_ensemble_download(sdg_ensemble* e, int i, double* q) {
  if (!e || i < 0 || i >= e->n || !q) return fail(SDG_ERR_INVALID_ARG, "bad ensemble download");
  const BatchInst& I = e->inst[i];
  const long long nd = (long long)(I.p + 1) * (I.p + 1) * (I.p + 1) * I.box.Ne;
  SDG_CUDA_TRY(cudaStreamSynchronize(e->stream));
  SDG_CUDA_TRY(cudaMemcpy(q, I.q[e->cur_host[i]], 8 * nd, cudaMemcpyDeviceToHost));
  return SDG_OK;
}

long long sdg_ensemble_total_dofs(const sdg_ensemble* e) { return e ? e->total_dof : 0; }

int sdg_ensemble_launches_per_step(const sdg_ensemble* e) {
  if (!e) return 0;
  return e->fj.fused ? 4 : 3 * (int)e->groups.size() + 1;
}

int sdg_ensemble_destroy(sdg_ensemble* e) {
  if (!e) return SDG_OK;
  free_ensemble(e);
  delete e;
  return SDG_OK;
}

}  // extern "C"
