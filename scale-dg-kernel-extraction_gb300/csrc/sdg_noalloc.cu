// Allocation-free variant of the device-pointer advection tendency.
//
// sdg_advect3d_eq_cal_tend_dev needs caller-owned scratch for the
// element-boundary flux (NfpTot*Ne doubles) and an error flag.  Some callers
// cannot obtain device memory at the point where they evaluate the tendency:
//   - a host model that reserves its whole HBM budget up front through its own
//     pool allocator, and has no headroom or API for ad-hoc allocations;
//   - a latency-bound request loop, where cudaMalloc/cudaFree would be
//     unacceptable because cudaFree synchronises the whole device and stalls
//     every other stream in flight;
//   - code that must not fail for lack of memory halfway through a time step.
// This entry point gives them the same computation with the scratch held in a
// fixed file-scope device array, so a call allocates nothing.
//
// Limits and sharing rules:
//   - the array holds kNoAllocFluxMax doubles (16 MiB); a call that needs more
//     (NfpTot*Ne larger than that) is rejected with SDG_ERR_INVALID_ARG;
//   - every GPU that loads the library holds the array until the process
//     exits;
//   - all calls on a device share the one array, which keeps whatever the last
//     call left in it.  The flux values are fully rewritten by every call; the
//     error flag is cleared at the start of every call.  Calls whose work
//     overlaps on the GPU (different streams, or different host threads on the
//     same device) race on the array and must be serialised by the caller;
//   - the device address of the array is resolved with cudaGetSymbolAddress
//     the first time the entry point runs on a device (with that device
//     current).  That first call should therefore come before any stream
//     capture.
#include <cuda_runtime.h>

#include <mutex>

#include "sdg_dropin.cuh"

namespace sdg {
// Launch path shared with sdg_advect3d_eq_cal_tend_dev (sdg_dropin.cu).
int tend_dev(const TendArgs& a, int p, int NfpTot, int opt, cudaStream_t st);
}  // namespace sdg

using namespace sdg;

namespace {

constexpr long long kNoAllocFluxMax = 1LL << 21;  // doubles, 16 MiB
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_flux[kNoAllocFluxMax];
static __device__ __align__(256) int g_noalloc_err;

struct NoAllocScratch {
  double* flux = nullptr;
  int* err = nullptr;
  bool ready = false;
};

std::mutex g_noalloc_mu;
NoAllocScratch g_noalloc_dev[kMaxDevices];

// Device addresses of the file-scope arrays for the current device.  In host
// code the array names are host-side stand-ins, never device addresses, so
// the kernels receive only what cudaGetSymbolAddress returns.
int noalloc_scratch(NoAllocScratch* out) {
  int dev = 0;
  SDG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices)
    return fail(SDG_ERR_INVALID_ARG, "device %d beyond the %d this entry point tracks", dev,
                kMaxDevices);
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  NoAllocScratch& s = g_noalloc_dev[dev];
  if (!s.ready) {
    void* f = nullptr;
    void* e = nullptr;
    SDG_CUDA_TRY(cudaGetSymbolAddress(&f, g_noalloc_flux));
    SDG_CUDA_TRY(cudaGetSymbolAddress(&e, g_noalloc_err));
    s.flux = static_cast<double*>(f);
    s.err = static_cast<int*>(e);
    s.ready = true;
  }
  *out = s;
  return SDG_OK;
}

}  // namespace

extern "C" int sdg_advect3d_eq_cal_tend_noalloc(
    double* dqdt, const double* q, const double* u, const double* v, const double* w,
    const double* D1D, const double* D1D_tr, const double* Lift_mat, const int* VMapM,
    const int* VMapP, const double* normal_fn, const double* Escale, const double* Fscale,
    int Nq, int Np, int NfpTot, int Ne, int NeA, int opt, void* stream) {
  if (opt != SDG_OPT_GENERAL && opt != SDG_OPT_OPT1 && opt != SDG_OPT_EVENODD)
    return fail(SDG_ERR_BAD_OPTTYPE, "unknown DGOptrKernel type %d", opt);
  if (Nq - 1 < 1 || Nq - 1 > kMaxOrder)
    return fail(SDG_ERR_UNSUPPORTED_ORDER, "PolyOrder %d outside 1..15", Nq - 1);
  if (Np != Nq * Nq * Nq || NfpTot != 6 * Nq * Nq || Ne < 0 || NeA < Ne)
    return fail(SDG_ERR_INVALID_ARG, "inconsistent sizes Nq=%d Np=%d NfpTot=%d Ne=%d NeA=%d",
                Nq, Np, NfpTot, Ne, NeA);
  const long long need = (long long)NfpTot * Ne;
  if (need > kNoAllocFluxMax)
    return fail(SDG_ERR_INVALID_ARG,
                "the allocation-free tendency holds at most %lld face-flux values "
                "(NfpTot*Ne); this call needs %lld -- use sdg_advect3d_eq_cal_tend_dev "
                "with caller-owned scratch",
                kNoAllocFluxMax, need);
  if (Ne == 0) return SDG_OK;
  if (!dqdt || !q || !u || !v || !w || !D1D || !D1D_tr || !Lift_mat || !VMapM || !VMapP ||
      !normal_fn || !Escale || !Fscale)
    return fail(SDG_ERR_INVALID_ARG, "NULL device pointer");
  SDG_TRY(require_device());
  NoAllocScratch sc;
  SDG_TRY(noalloc_scratch(&sc));
  cudaStream_t st = as_stream(stream);
  // the flag must start at zero; the flux scratch is fully overwritten
  SDG_CUDA_TRY(cudaMemsetAsync(sc.err, 0, sizeof(int), st));
  TendArgs a{dqdt, q, u, v, w, D1D, D1D_tr, Lift_mat, VMapM, VMapP, normal_fn,
             Escale, Fscale, sc.flux, sc.err, Ne, (long long)Np * NeA};
  SDG_TRY(tend_dev(a, Nq - 1, NfpTot, opt, st));
  int h_err = 0;
  SDG_CUDA_TRY(cudaMemcpyAsync(&h_err, sc.err, sizeof(int), cudaMemcpyDeviceToHost, st));
  SDG_CUDA_TRY(cudaStreamSynchronize(st));
  if (h_err == 2)
    return fail(SDG_ERR_INVALID_ARG,
                "D1D / D1D_tr / Lift_mat lack the even-odd symmetries; use GENERAL or OPT1");
  if (h_err) return fail(SDG_ERR_MESH, "a VMapM/VMapP entry is outside 1..Np*NeA");
  return SDG_OK;
}
