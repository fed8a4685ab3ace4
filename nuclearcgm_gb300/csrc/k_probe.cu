// FP64 pipe throughput probe: the denominator of the FP64 stencil's compute
// roofline. Every thread runs kChains independent chains of dependent FP64
// FMAs (enough independent work per warp to keep the pipe busy), on a grid of
// several CTAs per SM; the rate is counted as 2 flops per FMA.
#include "ncgm_internal.cuh"

#include <algorithm>

namespace ncgm {
namespace {

constexpr int kChains = 8;

__global__ void fp64FmaKernel(double *out, int iters, double a, double b) {
  double x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = threadIdx.x * 1e-9 + c;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], a, b);
  }
  double s = 0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += x[c];
  // keeps the chains live; written only for an impossible value
  if (s == -1.2345e300) out[blockIdx.x] = s;
}

} // namespace
} // namespace ncgm

using namespace ncgm;

// FP64 FMA throughput of the current device in GFLOP/s (2 flops per FMA),
// from CUDA events around one launch after a warm-up launch. A measurement
// helper for the FP64 forms' roofline; the reference has no counterpart.
extern "C" int ncgm_measure_fp64_gflops(double *gflops) {
  if (!gflops) {
    setError("ncgm_measure_fp64_gflops: null output");
    return NCGM_ERR_ARG;
  }
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
          cudaSuccess) {
    cudaGetLastError();
    setError("ncgm_measure_fp64_gflops: no CUDA device");
    return NCGM_ERR_CUDA;
  }
  const int blocks = sms * 8, threads = 256, iters = 1 << 14;
  double *out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  float ms = 0;
  cudaError_t e = cudaMalloc(&out, sizeof(double) * blocks);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess) {
    fp64FmaKernel<<<blocks, threads>>>(out, iters / 4, 0.999999, 1e-7);
    cudaEventRecord(e0);
    fp64FmaKernel<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(e1);
    e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (out) cudaFree(out);
  if (e != cudaSuccess || !(ms > 0)) {
    setError(std::string("ncgm_measure_fp64_gflops: ") +
             cudaGetErrorString(e));
    return NCGM_ERR_CUDA;
  }
  const double flops = 2.0 * kChains * (double)iters * threads * blocks;
  *gflops = flops / (ms * 1e-3) / 1e9;
  return NCGM_OK;
}
