// Throughput microbenchmarks of the arithmetic pipes the stage kernels use:
// DFMA, FFMA and the FP64<->FP32 conversions.  Each thread runs 8
// independent FMA chains so that the pipe, not the dependency latency, is the
// limit; the grid fills every SM several times over.
#include <cuda_runtime.h>

#include <chrono>

#include "sdg_internal.h"

using namespace sdg;

namespace {

template <typename T>
__global__ void fma_chain_kernel(T* out, int iters, T a, T b) {
  T x[8];
#pragma unroll
  for (int c = 0; c < 8; c++) x[c] = (T)(threadIdx.x + c);
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int c = 0; c < 8; c++) x[c] = fma(x[c], a, b);
  }
  T s = 0;
#pragma unroll
  for (int c = 0; c < 8; c++) s += x[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// Round trips double -> float -> double; the FP32 value is perturbed by an
// FP32 add so that the chain cannot be folded.
__global__ void cvt_chain_kernel(double* out, int iters, float c) {
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; k++) x[k] = (double)(threadIdx.x + k);
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = (double)((float)x[k] + c);
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename Launch>
int time_ms(Launch launch, float* ms) {
  cudaEvent_t e0, e1;
  SDG_CUDA_TRY(cudaEventCreate(&e0));
  SDG_CUDA_TRY(cudaEventCreate(&e1));
  launch();  // warm-up
  SDG_CUDA_TRY(cudaGetLastError());
  SDG_CUDA_TRY(cudaEventRecord(e0));
  launch();
  SDG_CUDA_TRY(cudaEventRecord(e1));
  SDG_CUDA_TRY(cudaEventSynchronize(e1));
  SDG_CUDA_TRY(cudaEventElapsedTime(ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return SDG_OK;
}

// Picks an iteration count that makes the timed launch last ~30 ms.
template <typename MakeLaunch>
int calibrated(MakeLaunch make, double ops_per_iter, double* rate) {
  int iters = 64;
  float ms = 0.f;
  for (int round = 0; round < 12; round++) {
    SDG_TRY(time_ms(make(iters), &ms));
    if (ms > 20.f || iters >= (1 << 22)) break;
    const double scale = (ms > 0.05f) ? 30.0 / ms : 16.0;
    iters = (int)(iters * (scale > 16.0 ? 16.0 : scale)) + 1;
  }
  *rate = ops_per_iter * iters / (ms * 1e-3);
  return SDG_OK;
}

}  // namespace

extern "C" int sdg_microbench_peaks(double* dfma_tflops, double* ffma_tflops,
                                    double* cvt_f64_f32_tops,
                                    double* cvt_f32_f64_tops) {
  SDG_TRY(require_device());
  int dev = 0, nsm = 0;
  SDG_CUDA_TRY(cudaGetDevice(&dev));
  SDG_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int threads = 256, blocks = nsm * 8;
  const double nthr = (double)threads * blocks;
  void* buf = nullptr;
  SDG_CUDA_TRY(cudaMalloc(&buf, sizeof(double) * threads * blocks));
  double r = 0;
  int st = SDG_OK;
  if (dfma_tflops && st == SDG_OK) {
    st = calibrated([&](int it) { return [=] {
      fma_chain_kernel<double><<<blocks, threads>>>((double*)buf, it, 0.999999, 1e-7); }; },
                    nthr * 8, &r);
    *dfma_tflops = 2.0 * r / 1e12;
  }
  if (ffma_tflops && st == SDG_OK) {
    st = calibrated([&](int it) { return [=] {
      fma_chain_kernel<float><<<blocks, threads>>>((float*)buf, it, 0.999f, 1e-3f); }; },
                    nthr * 8, &r);
    *ffma_tflops = 2.0 * r / 1e12;
  }
  if ((cvt_f64_f32_tops || cvt_f32_f64_tops) && st == SDG_OK) {
    st = calibrated([&](int it) { return [=] {
      cvt_chain_kernel<<<blocks, threads>>>((double*)buf, it, 1e-3f); }; },
                    nthr * 8, &r);
    // one round trip = one conversion each way (plus one FP32 add)
    if (cvt_f64_f32_tops) *cvt_f64_f32_tops = r / 1e12;
    if (cvt_f32_f64_tops) *cvt_f32_f64_tops = r / 1e12;
  }
  cudaFree(buf);
  return st;
}
