// peak.cu -- scft_fp64_fma_rate: the FP64 FMA throughput of the current GPU,
// measured, so that the plain FP64 method's kernels can be placed against an
// FP64 roofline as well as the HBM one (the measured peaks cover copy
// bandwidth and bf16 tensor throughput only).
//
// Each thread runs kChains independent FMA chains of kIters steps in
// registers (no memory traffic), on a grid of kBlocksPerSm CTAs of 256 threads
// per SM; the result is stored only so that the compiler keeps the chains.
// Timed with CUDA events on a private stream after one untimed launch.  No
// clock or other device setting is touched.
#include <cuda_runtime.h>

#include <string>

#include "../../include/scft.h"

namespace scft {

namespace {

constexpr int kChains = 8;
constexpr int kIters = 4096;
constexpr int kBlocksPerSm = 8;
constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) k_fp64_fma(double *out, double a, double b) {
  double x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; c++) x[c] = (double)(threadIdx.x + c);
  for (int i = 0; i < kIters; i++) {
#pragma unroll
    for (int c = 0; c < kChains; c++) x[c] = fma(x[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; c++) s += x[c];
  if (s == 1.2345) out[blockIdx.x] = s;  // never true for these inputs; keeps the chains live
}

}  // namespace

int fp64_fma_rate(int reps, double *gflops, std::string &msg) {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  double *out = nullptr;
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  const int blocks = sms * kBlocksPerSm;
  if (e == cudaSuccess) e = cudaMalloc(&out, sizeof(double) * (blocks > 0 ? blocks : 1));
  float ms = 0.f;
  if (e == cudaSuccess) {
    // a, b keep x bounded (|a| < 1) and the result away from 1.2345
    k_fp64_fma<<<blocks, kThreads, 0, st>>>(out, 0.999999, 1e-7);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaEventRecord(e0, st);
  for (int r = 0; r < reps && e == cudaSuccess; r++) {
    k_fp64_fma<<<blocks, kThreads, 0, st>>>(out, 0.999999, 1e-7);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaEventRecord(e1, st);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  if (out) cudaFree(out);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  if (e != cudaSuccess) {
    msg = std::string("CUDA: ") + cudaGetErrorString(e);
    return SCFT_ERR_CUDA;
  }
  const double flops = 2.0 * kChains * (double)kIters * kThreads * (double)blocks * reps;
  *gflops = flops / (ms * 1e-3) / 1e9;
  return SCFT_OK;
}

}  // namespace scft
