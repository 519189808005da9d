// Serving loop for advection solves (sdg_server_* in include/sdg_advect.h).
//
// Continuous batching: a scheduler thread owns the GPU.  Submitted requests
// wait in a queue; between steps the scheduler admits as many as the HBM
// budget and the slot count allow (state allocated stream-ordered from the
// CUDA memory pool, initial condition generated on the device), then advances
// EVERY active request by one SSP-RK3 step with the batched persistent
// kernel (three stage launches + index advance), so requests that arrive
// while others run share the same launches.  A request that has done its
// nstep steps is finished at once: optional copy of its final state to the
// caller's buffer, memory returned to the pool, waiters notified, latency
// (finish - submit, host steady clock) recorded.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "sdg_batch.cuh"
#include "sdg_internal.h"

using namespace sdg;

namespace {

using Clock = std::chrono::steady_clock;

struct Req {
  uint64_t ticket = 0;
  sdg_request r{};
  double* out = nullptr;  // caller buffer for the final state, may be null
  Clock::time_point t_submit, t_admit, t_done;
  void* mem = nullptr;
  size_t bytes = 0;
  BatchInst inst{};
  int steps_done = 0;
  int status = SDG_OK;
  bool done = false;
};

}  // namespace

struct sdg_server {
  sdg_server_config cfg{};
  float* d_ops[kBatchMaxOrder + 1][3] = {};  // D1D, Lift, even-odd tables (FP32)
  double* d_x1D[kBatchMaxOrder + 1] = {};
  cudaStream_t stream = nullptr;
  cudaMemPool_t pool = nullptr;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Req*> pending;
  std::vector<Req*> active;
  std::map<uint64_t, Req*> all;
  uint64_t next_ticket = 1;
  bool stop = false;
  std::thread worker;
  size_t bytes_in_use = 0;
  // device tables for the active set
  BatchInst* d_inst = nullptr;
  int d_inst_cap = 0;
  BatchItem* d_items = nullptr;
  int d_items_cap = 0;
  int n_items = 0;
  std::vector<BatchGroup> groups;  // one persistent launch per order active
  BatchForkJoin fj;                // a side stream per group
  int threads[kBatchMaxOrder + 1] = {};
  int epb[kBatchMaxOrder + 1] = {};
  // statistics
  std::vector<double> latencies;
  long long completed = 0, steps_run = 0, launches = 0;
  double dof_updates = 0.0;
  Clock::time_point t_first_submit{}, t_last_done{};
  bool any_submit = false;
  int fatal = SDG_OK;
  // host-side fault injection (sdg_server_inject_rebuild_failure): the next
  // table rebuild after a completion reports an allocation failure
  bool inject_on_completion = false;
  bool inject_rebuild_failure = false;
};

namespace {

size_t request_bytes(const sdg_request& r) {
  const long long np = (long long)(r.p + 1) * (r.p + 1) * (r.p + 1);
  const long long nd = np * r.NeX * r.NeY * r.NeZ;
  return (size_t)nd * (3 * 8 + 3 * 4);
}

long long request_dofs(const sdg_request& r) {
  return (long long)(r.p + 1) * (r.p + 1) * (r.p + 1) * r.NeX * r.NeY * r.NeZ;
}

int admit(sdg_server* s, Req* q) {
  const size_t bytes = request_bytes(q->r);
  void* mem = nullptr;
  SDG_CUDA_TRY(cudaMallocFromPoolAsync(&mem, bytes, s->pool, s->stream));
  q->mem = mem;
  q->bytes = bytes;
  const long long nd = request_dofs(q->r);
  BatchInst& I = q->inst;
  I.box = make_box(q->r.NeX, q->r.NeY, q->r.NeZ, 1.0, 1.0, 1.0);
  char* base = static_cast<char*>(mem);
  for (int k = 0; k < 3; k++) I.q[k] = reinterpret_cast<double*>(base + 8 * nd * k);
  float* vel = reinterpret_cast<float*>(base + 24 * nd);
  I.u = vel;
  I.v = vel + nd;
  I.w = vel + 2 * nd;
  I.p = q->r.p;
  I.D = s->d_ops[q->r.p][0];
  I.Lift = s->d_ops[q->r.p][1];
  I.eo_tab = s->d_ops[q->r.p][2];
  // opt 0: the measured default body of the order; EVENODD: even-odd everywhere
  I.eo = (I.eo_tab != nullptr && (s->cfg.opt != 0 || batch_default_eo(I.p))) ? 1 : 0;
  I.dt = q->r.dt;
  batch_stage_factors(I);
  I.cur = 0;
  I.active = 1;
  SDG_TRY(batch_init_blob(I, s->d_x1D[q->r.p], q->r.centre, q->r.sigma, q->r.velocity,
                          s->stream));
  q->t_admit = Clock::now();
  return SDG_OK;
}

// Rebuilds the instance table and the work items of the active set.
int rebuild_tables(sdg_server* s) {
  const int n = (int)s->active.size();
  std::vector<BatchInst> inst(n);
  std::vector<BatchItem> items;
  std::vector<int> order(n);
  for (int i = 0; i < n; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return s->active[a]->r.p > s->active[b]->r.p; });
  for (int i = 0; i < n; i++) {
    inst[i] = s->active[i]->inst;
    inst[i].cur = s->active[i]->steps_done % 3;
  }
  for (int i : order) {
    const BatchInst& I = inst[i];
    const int e = s->epb[I.p];
    for (long long b = 0; b < I.box.Ne; b += e)
      items.push_back({i, (int)b, (int)std::min<long long>(e, I.box.Ne - b),
                       2 * I.p + (I.eo ? 1 : 0)});
  }
  // grow a table only once its new allocation has succeeded, so that a
  // failed allocation leaves the old table and its capacity consistent
  if (s->inject_rebuild_failure) {
    s->inject_rebuild_failure = false;
    return fail(SDG_ERR_OUT_OF_MEMORY, "table rebuild failed (injected)");
  }
  if (n > s->d_inst_cap) {
    const int cap = std::max(n, 2 * s->d_inst_cap);
    BatchInst* t = nullptr;
    SDG_CUDA_TRY(cudaMalloc(&t, sizeof(BatchInst) * cap));
    cudaFree(s->d_inst);
    s->d_inst = t;
    s->d_inst_cap = cap;
  }
  if ((int)items.size() > s->d_items_cap) {
    const int cap = std::max((int)items.size(), 2 * s->d_items_cap);
    BatchItem* t = nullptr;
    SDG_CUDA_TRY(cudaMalloc(&t, sizeof(BatchItem) * cap));
    cudaFree(s->d_items);
    s->d_items = t;
    s->d_items_cap = cap;
  }
  if (n)
    SDG_CUDA_TRY(cudaMemcpyAsync(s->d_inst, inst.data(), sizeof(BatchInst) * n,
                                 cudaMemcpyHostToDevice, s->stream));
  if (!items.empty())
    SDG_CUDA_TRY(cudaMemcpyAsync(s->d_items, items.data(), sizeof(BatchItem) * items.size(),
                                 cudaMemcpyHostToDevice, s->stream));
  // the host vectors must outlive the asynchronous copies
  SDG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  s->n_items = (int)items.size();
  return batch_groups(items, inst, s->epb, s->threads, s->groups);
}

int run_steps(sdg_server* s, int nsteps) {
  const int n = (int)s->active.size();
  for (int k = 0; k < nsteps; k++) {
    SDG_TRY(batch_step_enqueue(s->fj, s->d_inst, n, s->d_items, s->groups, s->stream));
    s->launches += 3 * (long long)s->groups.size() + 1;
  }
  return SDG_OK;
}

void finish(sdg_server* s, Req* q, int status) {
  q->status = status;
  q->done = true;
  q->t_done = Clock::now();
  if (q->mem) {
    cudaFreeAsync(q->mem, s->stream);
    q->mem = nullptr;
    s->bytes_in_use -= q->bytes;
  }
}

// A failure that leaves the active set without usable tables (a failed step,
// a failed table rebuild): every active request finishes with the status,
// its memory goes back to the pool, and the server records the status.  The
// scheduler then launches nothing until new requests are admitted.
void fail_active(sdg_server* s, int st) {
  s->fatal = st;
  for (Req* q : s->active) finish(s, q, st);
  s->active.clear();
  s->n_items = 0;
  s->groups.clear();
  s->cv_done.notify_all();
}

void worker_loop(sdg_server* s) {
  cudaSetDevice(s->cfg.device);
  std::unique_lock<std::mutex> lk(s->mu);
  while (true) {
    // admission: as many queued requests as slots and the HBM budget allow
    bool changed = false;
    while (!s->pending.empty() && (int)s->active.size() < s->cfg.max_active) {
      Req* q = s->pending.front();
      if (s->bytes_in_use + request_bytes(q->r) > s->cfg.hbm_budget_bytes) {
        if (s->active.empty() && s->bytes_in_use == 0) {
          // larger than the whole budget: it can never run
          s->pending.pop_front();
          finish(s, q, SDG_ERR_OUT_OF_MEMORY);
          s->cv_done.notify_all();
          continue;
        }
        break;
      }
      s->pending.pop_front();
      const int st = admit(s, q);
      if (st != SDG_OK) {
        finish(s, q, st);
        s->cv_done.notify_all();
        continue;
      }
      s->bytes_in_use += q->bytes;
      s->active.push_back(q);
      changed = true;
    }
    if (s->active.empty()) {
      if (s->stop) break;
      s->cv_work.wait_for(lk, std::chrono::milliseconds(50));
      continue;
    }
    if (changed) {
      const int st = rebuild_tables(s);
      if (st != SDG_OK) {
        fail_active(s, st);
        continue;
      }
    }
    // run until the next request finishes, at most `window` steps so that new
    // arrivals wait for at most one window before admission
    int k = s->cfg.max_window_steps > 0 ? s->cfg.max_window_steps : 8;
    for (Req* q : s->active) k = std::min(k, q->r.nstep - q->steps_done);
    if (k < 1) k = 1;
    long long dofs = 0;
    for (Req* q : s->active) dofs += request_dofs(q->r);
    lk.unlock();
    int st = run_steps(s, k);
    if (st == SDG_OK) {
      cudaError_t ce = cudaStreamSynchronize(s->stream);
      if (ce != cudaSuccess) st = cuda_fail(ce, "server step", __FILE__, __LINE__);
    }
    lk.lock();
    s->steps_run += k;
    s->dof_updates += 3.0 * (double)dofs * k;
    if (st != SDG_OK) {
      fail_active(s, st);
      continue;
    }
    std::vector<Req*> still, done;
    for (Req* q : s->active) {
      q->steps_done += k;
      (q->steps_done >= q->r.nstep ? done : still).push_back(q);
    }
    const bool any_done = !done.empty();
    // result copies run without the lock, so that submitters and waiters are
    // not held up by them; only this thread touches a request's buffers
    std::vector<int> fst(done.size(), SDG_OK);
    lk.unlock();
    for (size_t i = 0; i < done.size(); i++) {
      Req* q = done[i];
      if (!q->out) continue;
      const long long nd = request_dofs(q->r);
      cudaError_t ce = cudaMemcpyAsync(q->out, q->inst.q[q->steps_done % 3], 8 * nd,
                                       cudaMemcpyDeviceToHost, s->stream);
      if (ce == cudaSuccess) ce = cudaStreamSynchronize(s->stream);
      if (ce != cudaSuccess) fst[i] = cuda_fail(ce, "result copy", __FILE__, __LINE__);
    }
    lk.lock();
    for (size_t i = 0; i < done.size(); i++) {
      Req* q = done[i];
      finish(s, q, fst[i]);
      s->completed++;
      s->latencies.push_back(std::chrono::duration<double>(q->t_done - q->t_submit).count());
      s->t_last_done = q->t_done;
    }
    if (any_done) {
      s->active.swap(still);
      if (!s->active.empty()) {
        // the old tables still point at the instances just freed: if they
        // cannot be rebuilt, no further step may run on them
        if (s->inject_on_completion) {
          s->inject_on_completion = false;
          s->inject_rebuild_failure = true;
        }
        const int rst = rebuild_tables(s);
        if (rst != SDG_OK) fail_active(s, rst);
      }
      s->cv_done.notify_all();
    }
  }
}

double percentile(std::vector<double> v, double pct) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  const double pos = pct / 100.0 * (double)(v.size() - 1);
  const size_t i = (size_t)pos;
  const double f = pos - (double)i;
  return (i + 1 < v.size()) ? v[i] * (1.0 - f) + v[i + 1] * f : v[i];
}

}  // namespace

extern "C" {

int sdg_server_create(sdg_server** out, const sdg_server_config* cfg,
                      const double* const* D1D_by_order, const double* const* Lift_by_order,
                      const double* const* x1D_by_order) {
  if (!out || !cfg || !D1D_by_order || !Lift_by_order || !x1D_by_order)
    return fail(SDG_ERR_INVALID_ARG, "NULL argument");
  *out = nullptr;
  if (cfg->max_active < 1 || cfg->hbm_budget_bytes == 0)
    return fail(SDG_ERR_INVALID_ARG, "server needs at least one slot and a budget");
  if (cfg->opt != 0 && cfg->opt != SDG_OPT_GENERAL && cfg->opt != SDG_OPT_OPT1 &&
      cfg->opt != SDG_OPT_EVENODD)
    return fail(SDG_ERR_BAD_OPTTYPE, "unknown opt type %d", cfg->opt);
  for (int p = -1; p < 16; p++) {
    const int t = p < 0 ? cfg->threads : cfg->threads_by_order[p];
    if (t != 0 && (t < 32 || t > kBatchThreadsMax || t % 32))
      return fail(SDG_ERR_INVALID_ARG, "bad block size %d", t);
  }
  SDG_TRY(require_device());
  sdg_server* s = new (std::nothrow) sdg_server();
  if (!s) return fail(SDG_ERR_OUT_OF_MEMORY, "host allocation failed");
  s->cfg = *cfg;
  s->fj.parallel = (cfg->parallel_groups != 0);
  for (int p = 0; p <= kBatchMaxOrder; p++) {
    batch_default_shape(p, &s->threads[p], &s->epb[p]);
    if (cfg->threads > 0) s->threads[p] = cfg->threads;
    if (cfg->threads_by_order[p] > 0) s->threads[p] = cfg->threads_by_order[p];
    if (cfg->epb_by_order[p] > 0) s->epb[p] = cfg->epb_by_order[p];
  }
  auto bail = [&](int st) {
    for (int p = 0; p <= kBatchMaxOrder; p++) {
      cudaFree(s->d_ops[p][0]);
      cudaFree(s->d_ops[p][1]);
      cudaFree(s->d_ops[p][2]);
      cudaFree(s->d_x1D[p]);
    }
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return st;
  };
  cudaError_t ce = cudaSetDevice(cfg->device);
  if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (ce == cudaSuccess) ce = cudaDeviceGetDefaultMemPool(&s->pool, cfg->device);
  if (ce == cudaSuccess) {
    // keep freed request memory in the pool for the next admission
    uint64_t thresh = UINT64_MAX;
    ce = cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &thresh);
  }
  if (ce == cudaSuccess) {
    // admission by free HBM: never promise more than 90% of what is free now
    size_t free_b = 0, total_b = 0;
    ce = cudaMemGetInfo(&free_b, &total_b);
    if (ce == cudaSuccess && s->cfg.hbm_budget_bytes > free_b / 10 * 9)
      s->cfg.hbm_budget_bytes = free_b / 10 * 9;
  }
  for (int p = 1; p <= kBatchMaxOrder && ce == cudaSuccess; p++) {
    if (!D1D_by_order[p] || !Lift_by_order[p] || !x1D_by_order[p]) continue;
    const int nq = p + 1, nd = nq * nq, nl = 6 * nq * nq * nq;
    std::vector<float> d(nd), l(nl);
    for (int k = 0; k < nd; k++) d[k] = (float)D1D_by_order[p][k];
    for (int k = 0; k < nl; k++) l[k] = (float)Lift_by_order[p][k];
    ce = cudaMalloc(&s->d_ops[p][0], 4 * nd);
    if (ce == cudaSuccess) ce = cudaMalloc(&s->d_ops[p][1], 4 * nl);
    if (ce == cudaSuccess) ce = cudaMalloc(&s->d_x1D[p], 8 * nq);
    if (ce == cudaSuccess) ce = cudaMemcpy(s->d_ops[p][0], d.data(), 4 * nd, cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(s->d_ops[p][1], l.data(), 4 * nl, cudaMemcpyHostToDevice);
    if (ce == cudaSuccess)
      ce = cudaMemcpy(s->d_x1D[p], x1D_by_order[p], 8 * nq, cudaMemcpyHostToDevice);
    // even-odd tables (opt 0 or EVENODD) when the operators have the symmetry
    std::vector<double> eo;
    const bool want_eo = (cfg->opt == 0 || cfg->opt == SDG_OPT_EVENODD);
    if (ce == cudaSuccess && want_eo &&
        eo_tables(nq, D1D_by_order[p], Lift_by_order[p], eo) == SDG_OK) {
      std::vector<float> ef(eo.begin(), eo.end());
      ce = cudaMalloc(&s->d_ops[p][2], 4 * ef.size());
      if (ce == cudaSuccess)
        ce = cudaMemcpy(s->d_ops[p][2], ef.data(), 4 * ef.size(), cudaMemcpyHostToDevice);
    }
  }
  if (ce != cudaSuccess) return bail(cuda_fail(ce, "server setup", __FILE__, __LINE__));
  try {
    s->worker = std::thread(worker_loop, s);
  } catch (...) {
    return bail(fail(SDG_ERR_INVALID_ARG, "cannot start the scheduler thread"));
  }
  *out = s;
  return SDG_OK;
}

int sdg_server_submit(sdg_server* s, const sdg_request* r, double* out_state, uint64_t* ticket) {
  if (!s || !r || !ticket) return fail(SDG_ERR_INVALID_ARG, "NULL argument");
  if (r->p < 1 || r->p > kBatchMaxOrder)
    return fail(SDG_ERR_UNSUPPORTED_ORDER, "order %d outside 1..%d", r->p, kBatchMaxOrder);
  if (r->NeX < 1 || r->NeY < 1 || r->NeZ < 1 || r->nstep < 1 || !(r->dt > 0) || !(r->sigma > 0))
    return fail(SDG_ERR_INVALID_ARG, "bad request");
  if (!s->d_ops[r->p][0])
    return fail(SDG_ERR_INVALID_ARG, "the server has no operators for order %d", r->p);
  Req* q = new (std::nothrow) Req();
  if (!q) return fail(SDG_ERR_OUT_OF_MEMORY, "host allocation failed");
  q->r = *r;
  q->out = out_state;
  q->t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) {
      delete q;
      return fail(SDG_ERR_INVALID_ARG, "server is shutting down");
    }
    q->ticket = s->next_ticket++;
    if (!s->any_submit) {
      s->any_submit = true;
      s->t_first_submit = q->t_submit;
    }
    s->all[q->ticket] = q;
    s->pending.push_back(q);
  }
  s->cv_work.notify_one();
  *ticket = q->ticket;
  return SDG_OK;
}

int sdg_server_wait(sdg_server* s, uint64_t ticket, double timeout_s, sdg_result* res) {
  if (!s) return fail(SDG_ERR_INVALID_ARG, "NULL server");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->all.find(ticket);
  if (it == s->all.end()) return fail(SDG_ERR_INVALID_ARG, "unknown ticket %llu",
                                      (unsigned long long)ticket);
  Req* q = it->second;
  const auto deadline = Clock::now() + std::chrono::duration_cast<Clock::duration>(
                                           std::chrono::duration<double>(timeout_s));
  while (!q->done) {
    if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && !q->done)
      return fail(SDG_ERR_TIMEOUT, "request %llu not finished within %.3f s",
                  (unsigned long long)ticket, timeout_s);
  }
  if (res) {
    res->status = q->status;
    res->latency_s = std::chrono::duration<double>(q->t_done - q->t_submit).count();
    res->queue_s = q->t_admit.time_since_epoch().count()
                       ? std::chrono::duration<double>(q->t_admit - q->t_submit).count()
                       : 0.0;
    res->dofs = request_dofs(q->r);
  }
  const int st = q->status;
  s->all.erase(it);
  delete q;
  if (st != SDG_OK) return fail(st, "request %llu failed", (unsigned long long)ticket);
  return SDG_OK;
}

int sdg_server_get_stats(sdg_server* s, sdg_server_stats* out) {
  if (!s || !out) return fail(SDG_ERR_INVALID_ARG, "NULL argument");
  std::lock_guard<std::mutex> lk(s->mu);
  out->completed = s->completed;
  out->active = (int)s->active.size();
  out->pending = (int)s->pending.size();
  out->steps_run = s->steps_run;
  out->launches = s->launches;
  out->dof_updates = s->dof_updates;
  out->bytes_in_use = s->bytes_in_use;
  out->p50_latency_s = percentile(s->latencies, 50.0);
  out->p99_latency_s = percentile(s->latencies, 99.0);
  out->span_s = s->completed ? std::chrono::duration<double>(s->t_last_done - s->t_first_submit)
                                   .count()
                             : 0.0;
  out->fatal_status = s->fatal;
  return SDG_OK;
}

int sdg_server_inject_rebuild_failure(sdg_server* s) {
  if (!s) return fail(SDG_ERR_INVALID_ARG, "NULL server");
  std::lock_guard<std::mutex> lk(s->mu);
  s->inject_on_completion = true;
  return SDG_OK;
}

int sdg_server_reset_stats(sdg_server* s) {
  if (!s) return fail(SDG_ERR_INVALID_ARG, "NULL server");
  std::lock_guard<std::mutex> lk(s->mu);
  s->latencies.clear();
  s->completed = s->steps_run = s->launches = 0;
  s->dof_updates = 0.0;
  s->any_submit = false;
  return SDG_OK;
}

int sdg_server_destroy(sdg_server* s) {
  if (!s) return SDG_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    // queued requests that never started are cancelled
    for (Req* q : s->pending) {
      q->status = SDG_ERR_INVALID_ARG;
      q->done = true;
      q->t_done = Clock::now();
    }
    s->pending.clear();
  }
  s->cv_work.notify_all();
  if (s->worker.joinable()) s->worker.join();
  s->cv_done.notify_all();
  cudaStreamSynchronize(s->stream);
  for (auto& kv : s->all) {
    if (kv.second->mem) cudaFreeAsync(kv.second->mem, s->stream);
    delete kv.second;
  }
  cudaStreamSynchronize(s->stream);
  for (int p = 0; p <= kBatchMaxOrder; p++) {
    cudaFree(s->d_ops[p][0]);
    cudaFree(s->d_ops[p][1]);
    cudaFree(s->d_ops[p][2]);
    cudaFree(s->d_x1D[p]);
  }
  cudaFree(s->d_inst);
  cudaFree(s->d_items);
  cudaStreamDestroy(s->stream);
  delete s;
  return SDG_OK;
}

}  // extern "C"
