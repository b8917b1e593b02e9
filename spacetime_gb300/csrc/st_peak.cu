// st_peak.cu -- measured FP32 fused-multiply-add ceiling of the device, the
// denominator of the trace kernel's roofline fraction (the kernel is bound by
// FP32 issue, not by memory or the tensor cores).
//
// Each thread runs 8 independent FMA chains (enough to cover the FMA pipe's
// latency at full occupancy) for `iters` iterations; the grid holds every SM
// at 2048 resident threads for a few hundred milliseconds.  The chains' sum
// is stored so nothing is eliminated.  Time: CUDA events on the stream.
#include <cuda_runtime.h>

#include "../../include/spacetime_gb300.h"

namespace {

constexpr int PEAK_THREADS = 256;
constexpr int PEAK_CHAINS = 8;

__global__ void __launch_bounds__(PEAK_THREADS) fma_peak_kernel(float* out, int iters, float a, float b) {
  float x[PEAK_CHAINS];
#pragma unroll
  for (int c = 0; c < PEAK_CHAINS; ++c) x[c] = (float)(threadIdx.x + c) * 1e-3f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
#pragma unroll
      for (int c = 0; c < PEAK_CHAINS; ++c) x[c] = fmaf(x[c], a, b);
    }
  }
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < PEAK_CHAINS; ++c) s += x[c];
  out[blockIdx.x * PEAK_THREADS + threadIdx.x] = s;
}

}  // namespace

extern "C" int st_measure_fp32_peak(int device, int iters, double* tflops, double* ms_out) {
  if (iters <= 0 || !tflops) return ST_EINVAL;
  if (cudaSetDevice(device) != cudaSuccess) return ST_ECUDA;
  int nsm = 0, per_sm = 0;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return ST_ECUDA;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fma_peak_kernel, PEAK_THREADS, 0) != cudaSuccess)
    return ST_ECUDA;
  if (per_sm < 1) per_sm = 1;
  const int blocks = nsm * per_sm;
  float* out = nullptr;
  if (cudaMalloc(&out, (size_t)blocks * PEAK_THREADS * sizeof(float)) != cudaSuccess) return ST_ENOMEM;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = ST_OK;
  float best = 0.f;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) rc = ST_ECUDA;
  // one untimed launch (clocks up, code resident), then the best of three
  for (int rep = 0; rep < 4 && rc == ST_OK; ++rep) {
    cudaEventRecord(e0, 0);
    fma_peak_kernel<<<blocks, PEAK_THREADS>>>(out, iters, 0.9999f, 1e-4f);
    cudaEventRecord(e1, 0);
    if (cudaGetLastError() != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) { rc = ST_ECUDA; break; }
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) { rc = ST_ECUDA; break; }
    if (rep > 0 && (best == 0.f || ms < best)) best = ms;
  }
  if (rc == ST_OK) {
    const double fmas = (double)blocks * PEAK_THREADS * (double)iters * 16.0 * PEAK_CHAINS;
    *tflops = 2.0 * fmas / (best * 1e-3) / 1e12;
    if (ms_out) *ms_out = best;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(out);
  return rc;
}
