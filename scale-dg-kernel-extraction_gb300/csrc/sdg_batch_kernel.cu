// The persistent batched stage kernel and its helpers (see sdg_batch.cuh).
#include "sdg_batch.cuh"

namespace sdg {

namespace {

// SSP-RK3 coefficients, mod_common.f90:28-30
__constant__ double c_rk_a[3] = {0.0, 0.75, 1.0 / 3.0};
__constant__ double c_rk_b[3] = {1.0, 0.25, 2.0 / 3.0};

// 32-bit words of an instance header, copied into shared memory by as many
// threads.
constexpr int kInstWords = (int)(sizeof(BatchInst) / 4);
static_assert(sizeof(BatchInst) % 4 == 0, "instance header is copied as 32-bit words");
static_assert(kInstWords < 128, "the smallest block must copy the header in one pass");

// One persistent launch runs the items of one order group (order P, stage
// body EO: 1 even-odd, 0 node body; RK the stage's update kind).  Compiling
// one order and one body per kernel keeps each at its own register count
// (32 or 40, for 4 or 3 blocks of 512 threads an SM), where a switch over
// the orders would keep the union of their needs.
//
// Items are assigned round-robin (block b runs items b, b + G, b + 2G, ...).
// The next item's instance header is fetched into shared memory while the
// current item computes, and the item after that into a register, so that a
// block never waits on the item -> instance -> data chain of dependent loads.
// Resident blocks of 512 threads an SM the registers are capped for: 4 (32
// registers) where that measured faster on GB300, else 3 (40 registers).
// The node body gains 4-16 % from the fourth block at every order; the
// even-odd body, in its one-item kernel, up to 15 % (p = 2, 3) at every order
// but p = 10 (0.92x there).
template <int P, int EO>
__host__ __device__ constexpr int batch_min_blocks() {
  return (EO != 0 && P == 10) ? 3 : 4;
}

// Even-odd body: F_y / F_z formed on the fly rather than staged at the orders
// where that measured faster in the batch on GB300 (1.05x at p = 6, 1.11x at
// p = 8; 0.96-0.97x at p = 10 and 11).
template <int P>
__host__ __device__ constexpr bool batch_eo_fly() {
  return P == 6 || P == 8;
}

// Even-odd body: threads a line.  One up to p = 4, where a line has at most
// two output pairs (measured in the batch on GB300: p = 3 81.5 against 75.3,
// p = 4 82.1 against 71.6 GDOF-updates/s), two above (one at p = 5 with 64
// registers measured 439 against 450 solves/s on the 256-member ensemble,
// and at p = 11 level on the serving stream).
template <int P>
__host__ __device__ constexpr int batch_eo_parts() {
  return P <= 4 ? 1 : 2;
}

// One work item through one stage: the instance's buffers for the stage from
// its current index, then the order's stage body.
template <int P, int EO, int RK>
__device__ __forceinline__ void batch_item_body(const BatchInst& I, const BatchItem& w,
                                                int stage, unsigned char* smem) {
  const int s0 = I.cur, s1 = (s0 + 1) % 3, s2 = (s0 + 2) % 3;
  StageArgs a;
  a.q_in = (stage == 0) ? I.q[s0] : (stage == 1) ? I.q[s1] : I.q[s2];
  a.q0 = (stage == 0) ? nullptr : I.q[s0];
  a.q_out = (stage == 1) ? I.q[s2] : I.q[s1];
  a.u = I.u;
  a.v = I.v;
  a.w = I.w;
  a.D = EO ? static_cast<const void*>(I.eo_tab) : static_cast<const void*>(I.D);
  a.Lift = I.Lift;
  a.box = I.box;
  a.fc_out = nullptr;
  a.fc_in = nullptr;
  a.elem_begin = 0;
  a.elem_count = I.box.Ne;
  a.a = c_rk_a[stage];
  a.b = c_rk_b[stage];
  a.dt = I.dt;
  a.cdt_hi = I.cdt[stage];  // FP32 increment factor of the FP32 form
  a.cdt_lo = 0.0f;
  a.b_is_one = (stage == 0);
  a.a_nonzero = (stage != 0);
  a.tend_only = 0;
  if constexpr (EO != 0) {
    for (int d = 0; d < 3; d++) {
      a.eo_sDf[d] = I.eo_sD[stage][d];
      a.eo_sLf[d] = I.eo_sL[stage][d];
    }
    stage_eo_block<P, float, RK, batch_eo_fly<P>(), false, batch_eo_parts<P>()>(
        a, w.e_begin, w.e_count, smem);
  } else {
    stage_block<P, float, float, false, RK>(a, w.e_begin, w.e_count, smem);
  }
}

// One block per work item, no loop: no work-item state stays live across
// the stage body, so the body keeps the registers the persistent form
// spends on its prefetch pipeline (the persistent kernel spilled 40-48 bytes
// at p = 7 under the 32-register cap).  Measured on GB300 for the even-odd
// body: 1.03-1.15x at every order but p = 8 (p = 7: 103.5 against 89.9
// GDOF-updates/s), 0.97x at p = 8; the node body is faster persistent.
template <int P, int EO>
__host__ __device__ constexpr bool batch_one_item() {
  return EO != 0 && P != 8;
}

template <int P, int EO, int RK>
__global__ void __launch_bounds__(kBatchThreadsMax, batch_min_blocks<P, EO>())
    batch_item_kernel(const BatchInst* __restrict__ insts, const BatchItem* __restrict__ items,
                      int n_items, int stage) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ __align__(16) BatchInst s_inst;
  __shared__ BatchItem s_item;
  const int tid = threadIdx.x;
  if ((int)blockIdx.x >= n_items) return;  // uniform across the block
  if (tid == 0) s_item = items[blockIdx.x];
  __syncthreads();
  if (tid < kInstWords)
    reinterpret_cast<uint32_t*>(&s_inst)[tid] =
        reinterpret_cast<const uint32_t*>(insts + s_item.inst)[tid];
  __syncthreads();
  if (s_inst.active) batch_item_body<P, EO, RK>(s_inst, s_item, stage, smem);
}

template <int P, int EO, int RK>
__global__ void __launch_bounds__(kBatchThreadsMax, batch_min_blocks<P, EO>())
    batch_order_kernel(const BatchInst* __restrict__ insts, const BatchItem* __restrict__ items,
                       int n_items, int stage) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ __align__(16) BatchInst s_inst[2];
  __shared__ BatchItem s_items[2];
  const int G = gridDim.x, tid = threadIdx.x;
  int it = blockIdx.x;
  if (it >= n_items) return;  // uniform across the block
  // prologue: the first item, its header, and the second item
  if (tid == 0) {
    s_items[0] = items[it];
    if (it + G < n_items) s_items[1] = items[it + G];
  }
  __syncthreads();
  if (tid < kInstWords)
    reinterpret_cast<uint32_t*>(&s_inst[0])[tid] =
        reinterpret_cast<const uint32_t*>(insts + s_items[0].inst)[tid];
  __syncthreads();

  for (int k = 0; it < n_items; k++, it += G) {
    const int slot = k & 1;
    const bool has_next = it + G < n_items, has_next2 = it + 2 * G < n_items;
    // prefetch, consumed after this item: the next item's header words and
    // the item after it
    uint32_t hw = 0;
    BatchItem nn{};
    if (has_next && tid < kInstWords)
      hw = reinterpret_cast<const uint32_t*>(insts + s_items[slot ^ 1].inst)[tid];
    if (has_next2 && tid == blockDim.x - 1) nn = items[it + 2 * G];

    const BatchItem w = s_items[slot];
    const BatchInst& I = s_inst[slot];
    if (I.active) batch_item_body<P, EO, RK>(I, w, stage, smem);
    // every read of this item's slots happened before the body's barriers
    __syncthreads();
    if (has_next && tid < kInstWords) reinterpret_cast<uint32_t*>(&s_inst[slot ^ 1])[tid] = hw;
    if (has_next2 && tid == blockDim.x - 1) s_items[slot] = nn;
    __syncthreads();  // the next item's header and the dynamic shared memory are ready
  }
}

// ONE persistent launch per RK stage over the work items of every order:
// blocks take items round-robin, read the item's instance header and run the
// stage body compiled for that instance's order and body (a switch over the
// 22 (order, body) pairs).  Block size and dynamic shared memory are the
// largest the present orders need; each body takes the block size at run
// time, so an item's bits are the per-order kernels'.  The kernel carries the
// register needs of every body at once (capped at 64 for two blocks of 512
// threads an SM), which is why the per-order launches are the default.
template <int RK>
__global__ void __launch_bounds__(kBatchThreadsMax, 2)
    batch_stage_kernel(const BatchInst* __restrict__ insts, const BatchItem* __restrict__ items,
                       int n_items, int stage) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ __align__(16) BatchInst s_inst;
  __shared__ BatchItem s_item;
  const int tid = threadIdx.x;
  for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
    __syncthreads();  // the previous item's readers of s_inst / smem are done
    if (tid == 0) s_item = items[it];
    __syncthreads();
    if (tid < kInstWords)
      reinterpret_cast<uint32_t*>(&s_inst)[tid] =
          reinterpret_cast<const uint32_t*>(insts + s_item.inst)[tid];
    __syncthreads();
    if (!s_inst.active) continue;  // uniform across the block
    // the body recorded in the item, which the groups' shared-memory sizes
    // were computed for (the device instance table's copy of the body flag
    // is not refreshed when the body changes)
    switch (s_item.body) {
#define SDG_FUSED_CASE(P)                                                    \
  case 2 * P: batch_item_body<P, 0, RK>(s_inst, s_item, stage, smem); break; \
  case 2 * P + 1: batch_item_body<P, 1, RK>(s_inst, s_item, stage, smem); break;
      SDG_FUSED_CASE(1) SDG_FUSED_CASE(2) SDG_FUSED_CASE(3) SDG_FUSED_CASE(4)
      SDG_FUSED_CASE(5) SDG_FUSED_CASE(6) SDG_FUSED_CASE(7) SDG_FUSED_CASE(8)
      SDG_FUSED_CASE(9) SDG_FUSED_CASE(10) SDG_FUSED_CASE(11)
#undef SDG_FUSED_CASE
      default: break;
    }
  }
}

__global__ void batch_advance_kernel(BatchInst* insts, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && insts[i].active) insts[i].cur = (insts[i].cur + 1) % 3;
}

__global__ void init_blob_kernel(double* q, float* u, float* v, float* w, const double* x1D,
                                 Box box, int nq, double cx, double cy, double cz,
                                 double inv2s2, float ux, float uy, float uz) {
  const long long np = (long long)nq * nq * nq;
  const long long total = np * box.Ne;
  const double dx = 2.0 / box.Es[0], dy = 2.0 / box.Es[1], dz = 2.0 / box.Es[2];
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    const long long e = g / np;
    const int n = (int)(g - e * np);
    const int i = n % nq, j = (n / nq) % nq, k = n / (nq * nq);
    const int ex = (int)(e % box.NeX);
    const int ey = (int)((e / box.NeX) % box.NeY);
    const int ez = (int)(e / ((long long)box.NeX * box.NeY));
    // node position as mesh_setup places it (mod_mesh.f90:141-145, :344-347)
    const double x = (ex + 0.5) * dx + 0.5 * dx * x1D[i];
    const double y = (ey + 0.5) * dy + 0.5 * dy * x1D[j];
    const double z = (ez + 0.5) * dz + 0.5 * dz * x1D[k];
    double ddx = x - cx, ddy = y - cy, ddz = z - cz;
    ddx -= rint(ddx);
    ddy -= rint(ddy);
    ddz -= rint(ddz);
    q[g] = exp(-(ddx * ddx + ddy * ddy + ddz * ddz) * inv2s2);
    u[g] = ux;
    v[g] = uy;
    w[g] = uz;
  }
}

template <int P>
size_t smem_for(int epb, int eo) {
  return eo ? eo_block_smem<P, float, batch_eo_fly<P>(), batch_eo_parts<P>()>(epb)
            : stage_block_smem<P, float>(epb);
}

}  // namespace

size_t batch_smem_bytes(int p, int epb, int eo) {
  switch (p) {
    case 1: return smem_for<1>(epb, eo);
    case 2: return smem_for<2>(epb, eo);
    case 3: return smem_for<3>(epb, eo);
    case 4: return smem_for<4>(epb, eo);
    case 5: return smem_for<5>(epb, eo);
    case 6: return smem_for<6>(epb, eo);
    case 7: return smem_for<7>(epb, eo);
    case 8: return smem_for<8>(epb, eo);
    case 9: return smem_for<9>(epb, eo);
    case 10: return smem_for<10>(epb, eo);
    case 11: return smem_for<11>(epb, eo);
    default: return 0;
  }
}

namespace {
// The three functions an order group needs, for one (P, EO) pair.
template <int P, int EO>
struct GroupOps {
  static constexpr bool kOneItem = batch_one_item<P, EO>();
  static int set_smem(size_t smem) {
    SDG_CUDA_TRY(cudaFuncSetAttribute(batch_order_kernel<P, EO, kRkFirst>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    SDG_CUDA_TRY(cudaFuncSetAttribute(batch_order_kernel<P, EO, kRkGeneral>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if constexpr (kOneItem) {
      SDG_CUDA_TRY(cudaFuncSetAttribute(batch_item_kernel<P, EO, kRkFirst>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      SDG_CUDA_TRY(cudaFuncSetAttribute(batch_item_kernel<P, EO, kRkGeneral>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    }
    return SDG_OK;
  }
  static int blocks_per_sm(int threads, size_t smem) {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batch_order_kernel<P, EO, kRkGeneral>,
                                                      threads, smem) != cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    return nb;
  }
  static int launch(const BatchInst* d_inst, const BatchItem* d_items, int n, int stage,
                    int grid, int threads, size_t smem, cudaStream_t st) {
    if constexpr (kOneItem) {
      if (stage == 0)
        batch_item_kernel<P, EO, kRkFirst><<<grid, threads, smem, st>>>(d_inst, d_items, n,
                                                                        stage);
      else
        batch_item_kernel<P, EO, kRkGeneral><<<grid, threads, smem, st>>>(d_inst, d_items, n,
                                                                          stage);
      SDG_CUDA_TRY(cudaGetLastError());
      return SDG_OK;
    }
    if (stage == 0)
      batch_order_kernel<P, EO, kRkFirst><<<grid, threads, smem, st>>>(d_inst, d_items, n, stage);
    else
      batch_order_kernel<P, EO, kRkGeneral><<<grid, threads, smem, st>>>(d_inst, d_items, n,
                                                                         stage);
    SDG_CUDA_TRY(cudaGetLastError());
    return SDG_OK;
  }
};

template <template <int, int> class OPS, typename F>
int with_group(int p, int eo, F&& f) {
  switch (p * 2 + (eo ? 1 : 0)) {
#define SDG_GROUP_CASE(P) \
  case 2 * P: return f(OPS<P, 0>{}); \
  case 2 * P + 1: return f(OPS<P, 1>{});
    SDG_GROUP_CASE(1) SDG_GROUP_CASE(2) SDG_GROUP_CASE(3) SDG_GROUP_CASE(4)
    SDG_GROUP_CASE(5) SDG_GROUP_CASE(6) SDG_GROUP_CASE(7) SDG_GROUP_CASE(8)
    SDG_GROUP_CASE(9) SDG_GROUP_CASE(10) SDG_GROUP_CASE(11)
#undef SDG_GROUP_CASE
    default: return fail(SDG_ERR_UNSUPPORTED_ORDER, "batched order %d outside 1..11", p);
  }
}
}  // namespace

void batch_default_shape(int p, int* threads, int* epb) {
  // index = order; measured with sdg_ensemble_tune, block sizes 128/256/512
  static const int kThreads[kBatchMaxOrder + 1] = {256, 128, 256, 256, 256, 256,
                                                   256, 512, 256, 256, 256, 512};
  static const int kEpb[kBatchMaxOrder + 1] = {1, 64, 32, 16, 8, 4, 4, 4, 2, 1, 1, 1};
  const int i = (p >= 1 && p <= kBatchMaxOrder) ? p : 0;
  *threads = kThreads[i];
  *epb = kEpb[i];
}

int batch_default_eo(int p) { return p >= 1 ? 1 : 0; }

int batch_group_setup(BatchGroup& g) {
  const int threads = g.threads;
  int dev = 0, nsm = 0;
  SDG_CUDA_TRY(cudaGetDevice(&dev));
  SDG_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  int per_sm = 0;
  bool one_item = false;
  const int st = with_group<GroupOps>(g.p, g.eo, [&](auto ops) {
    const int r = decltype(ops)::set_smem(g.smem);
    if (r != SDG_OK) return r;
    per_sm = decltype(ops)::blocks_per_sm(threads, g.smem);
    one_item = decltype(ops)::kOneItem;
    return SDG_OK;
  });
  if (st != SDG_OK) return st;
  if (per_sm <= 0)
    return fail(SDG_ERR_INVALID_ARG, "batch kernel of order %d does not fit: %d threads, %zu B",
                g.p, threads, g.smem);
  const long long cap = (long long)nsm * per_sm;
  g.grid = one_item ? g.count : (int)(g.count < cap ? g.count : cap);
  return SDG_OK;
}

int batch_group_launch(const BatchInst* d_inst, const BatchItem* d_items, const BatchGroup& g,
                       int stage, cudaStream_t st) {
  if (g.count <= 0) return SDG_OK;
  return with_group<GroupOps>(g.p, g.eo, [&](auto ops) {
    return decltype(ops)::launch(d_inst, d_items + g.begin, g.count, stage, g.grid, g.threads,
                                 g.smem, st);
  });
}

BatchForkJoin::~BatchForkJoin() {
  for (cudaStream_t s : streams) cudaStreamDestroy(s);
  for (cudaEvent_t e : done) cudaEventDestroy(e);
  if (fork) cudaEventDestroy(fork);
}

// The three stages as one persistent launch each over every group's items
// (they are contiguous, sorted by order and body), then the index advance.
static int batch_fused_enqueue(BatchInst* d_inst, int n_inst, const BatchItem* d_items,
                               const std::vector<BatchGroup>& groups, cudaStream_t st) {
  int n_items = 0, threads = 32;
  size_t smem = 0;
  for (const BatchGroup& g : groups) {
    n_items = g.begin + g.count > n_items ? g.begin + g.count : n_items;
    threads = g.threads > threads ? g.threads : threads;
    smem = g.smem > smem ? g.smem : smem;
  }
  if (n_items > 0) {
    SDG_TRY(set_kernel_smem((const void*)batch_stage_kernel<kRkFirst>, (int)smem, false));
    SDG_TRY(set_kernel_smem((const void*)batch_stage_kernel<kRkGeneral>, (int)smem, false));
    int dev = 0, nsm = 0, per_sm = 0;
    SDG_CUDA_TRY(cudaGetDevice(&dev));
    SDG_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    SDG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, batch_stage_kernel<kRkGeneral>, threads, smem));
    if (per_sm < 1)
      return fail(SDG_ERR_INVALID_ARG, "the single-launch stage kernel does not fit an SM "
                  "(%d threads, %zu bytes of shared memory)", threads, smem);
    const long long cap = (long long)nsm * per_sm;
    const int grid = (int)(n_items < cap ? n_items : cap);
    for (int s = 0; s < 3; s++) {
      if (s == 0)
        batch_stage_kernel<kRkFirst><<<grid, threads, smem, st>>>(d_inst, d_items, n_items, s);
      else
        batch_stage_kernel<kRkGeneral><<<grid, threads, smem, st>>>(d_inst, d_items, n_items, s);
      SDG_CUDA_TRY(cudaGetLastError());
    }
  }
  return batch_advance_launch(d_inst, n_inst, st);
}

int batch_step_enqueue(BatchForkJoin& fj, BatchInst* d_inst, int n_inst,
                       const BatchItem* d_items, const std::vector<BatchGroup>& groups,
                       cudaStream_t st) {
  if (fj.fused) return batch_fused_enqueue(d_inst, n_inst, d_items, groups, st);
  const size_t ng = groups.size();
  if (ng <= 1 || !fj.parallel) {
    for (int s = 0; s < 3; s++)
      for (const BatchGroup& g : groups) SDG_TRY(batch_group_launch(d_inst, d_items, g, s, st));
    return batch_advance_launch(d_inst, n_inst, st);
  }
  if (!fj.fork) SDG_CUDA_TRY(cudaEventCreateWithFlags(&fj.fork, cudaEventDisableTiming));
  while (fj.streams.size() < ng) {
    cudaStream_t s;
    cudaEvent_t e;
    SDG_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    fj.streams.push_back(s);
    SDG_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    fj.done.push_back(e);
  }
  SDG_CUDA_TRY(cudaEventRecord(fj.fork, st));
  for (size_t i = 0; i < ng; i++) {
    SDG_CUDA_TRY(cudaStreamWaitEvent(fj.streams[i], fj.fork, 0));
    for (int s = 0; s < 3; s++)
      SDG_TRY(batch_group_launch(d_inst, d_items, groups[i], s, fj.streams[i]));
    SDG_CUDA_TRY(cudaEventRecord(fj.done[i], fj.streams[i]));
    SDG_CUDA_TRY(cudaStreamWaitEvent(st, fj.done[i], 0));
  }
  return batch_advance_launch(d_inst, n_inst, st);
}

int batch_groups(const std::vector<BatchItem>& items, const std::vector<BatchInst>& inst,
                 const int* epb, const int* threads, std::vector<BatchGroup>& groups) {
  groups.clear();
  for (size_t i = 0; i < items.size();) {
    const BatchInst& I = inst[items[i].inst];
    BatchGroup g;
    g.p = I.p;
    g.eo = I.eo;
    g.begin = (int)i;
    size_t j = i;
    while (j < items.size() && inst[items[j].inst].p == g.p && inst[items[j].inst].eo == g.eo)
      j++;
    g.count = (int)(j - i);
    g.threads = threads[g.p];
    g.smem = batch_smem_bytes(g.p, epb[g.p], g.eo);
    g.grid = 0;
    SDG_TRY(batch_group_setup(g));
    groups.push_back(g);
    i = j;
  }
  return SDG_OK;
}

int batch_advance_launch(BatchInst* d_inst, int n_inst, cudaStream_t st) {
  if (n_inst <= 0) return SDG_OK;
  batch_advance_kernel<<<(n_inst + 255) / 256, 256, 0, st>>>(d_inst, n_inst);
  SDG_CUDA_TRY(cudaGetLastError());
  return SDG_OK;
}

int batch_init_blob(const BatchInst& inst, const double* d_x1D, const double centre[3],
                    double sigma, const double vel[3], cudaStream_t st) {
  const int nq = inst.p + 1;
  const long long total = (long long)nq * nq * nq * inst.box.Ne;
  long long nb = (total + 255) / 256;
  if (nb > 152LL * 32) nb = 152LL * 32;
  init_blob_kernel<<<(unsigned)(nb > 0 ? nb : 1), 256, 0, st>>>(
      inst.q[inst.cur], const_cast<float*>(inst.u), const_cast<float*>(inst.v),
      const_cast<float*>(inst.w), d_x1D, inst.box, nq, centre[0], centre[1], centre[2],
      1.0 / (2.0 * sigma * sigma), (float)vel[0], (float)vel[1], (float)vel[2]);
  SDG_CUDA_TRY(cudaGetLastError());
  return SDG_OK;
}

}  // namespace sdg
