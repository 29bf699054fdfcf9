// FP64 arithmetic rates of the device, measured: the FP64 FMA pipe and the
// FP64 tensor path (mma.sync m8n8k4 f64), each in a register-only loop over
// 8 blocks of 256 threads per SM, timed with CUDA events after one untimed
// run.  The sigma kernels and the Davidson vector algebra are bound by the
// first on this GPU; the second tells whether moving the tall-skinny
// projections to the FP64 tensor path would pay.
//
// A benchmark utility, not part of the engine: built into its own library
// (libsbdgb_rates.so) that only bench.py loads, to state the FP64 roof the
// sigma kernels are measured against.  Returns 0 on success, 3 on a CUDA error.
#include <cuda_runtime.h>

namespace {

constexpr int kRateThreads = 256, kRateIters = 4096;

__global__ void __launch_bounds__(kRateThreads) k_rate_dfma(double *out) {
  double a = 1.0 + threadIdx.x * 1e-9, b = 1.0 - threadIdx.x * 1e-9;
  double c[8] = {};
  for (int i = 0; i < kRateIters; ++i) {
#pragma unroll
    for (int u = 0; u < 8; ++u) c[u] = fma(a, b, c[u]);
  }
  double s = 0.0;
  for (int u = 0; u < 8; ++u) s += c[u];
  if (s == 12345.0) out[blockIdx.x] = s;  // never true: keeps the loop alive
}

__global__ void __launch_bounds__(kRateThreads) k_rate_dmma(double *out) {
  double a = 1.0 + threadIdx.x * 1e-9, b = 1.0 - threadIdx.x * 1e-9;
  double c[4][2] = {};
  for (int i = 0; i < kRateIters; ++i) {
#pragma unroll
    for (int u = 0; u < 4; ++u)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                   : "+d"(c[u][0]), "+d"(c[u][1])
                   : "d"(a), "d"(b));
  }
  double s = 0.0;
  for (int u = 0; u < 4; ++u) s += c[u][0] + c[u][1];
  if (s == 12345.0) out[blockIdx.x] = s;
}

// Both loops' work in one loop: the FP64 FMAs and the FP64 MMAs interleaved.
// Timed against the two loops alone, it tells whether the FMA pipe and the
// FP64 tensor path run concurrently (time near the longer one) or share the
// FP64 units (time near their sum).
__global__ void __launch_bounds__(kRateThreads) k_rate_both(double *out) {
  double a = 1.0 + threadIdx.x * 1e-9, b = 1.0 - threadIdx.x * 1e-9;
  double c[8] = {};
  double m[4][2] = {};
  for (int i = 0; i < kRateIters; ++i) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                   : "+d"(m[u][0]), "+d"(m[u][1])
                   : "d"(a), "d"(b));
      c[2 * u] = fma(a, b, c[2 * u]);
      c[2 * u + 1] = fma(a, b, c[2 * u + 1]);
    }
  }
  double s = 0.0;
  for (int u = 0; u < 8; ++u) s += c[u];
  for (int u = 0; u < 4; ++u) s += m[u][0] + m[u][1];
  if (s == 12345.0) out[blockIdx.x] = s;
}

}  // namespace

// Milliseconds of the FMA loop, the MMA loop and the interleaved loop (same
// work as both), each after one untimed run.  Returns 0, or 3 on a CUDA error.
extern "C" int sbdgb_measure_fp64_overlap(int device, float *ms_fma, float *ms_mma, float *ms_both) {
  if (!ms_fma || !ms_mma || !ms_both) return 1;
  int sms = 0;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
    cudaGetLastError();
    return 3;
  }
  const int blocks = sms * 8;
  double *out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = 0;
  if (cudaMalloc(&out, sizeof(double) * blocks) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
      cudaEventCreate(&e1) != cudaSuccess)
    rc = 3;
  float *dst[3] = {ms_fma, ms_mma, ms_both};
  for (int kind = 0; kind < 3 && rc == 0; ++kind)
    for (int rep = 0; rep < 2 && rc == 0; ++rep) {
      cudaEventRecord(e0, 0);
      if (kind == 0) k_rate_dfma<<<blocks, kRateThreads>>>(out);
      if (kind == 1) k_rate_dmma<<<blocks, kRateThreads>>>(out);
      if (kind == 2) k_rate_both<<<blocks, kRateThreads>>>(out);
      cudaEventRecord(e1, 0);
      if (cudaEventSynchronize(e1) != cudaSuccess) rc = 3;
      cudaEventElapsedTime(dst[kind], e0, e1);
    }
  if (rc == 0 && cudaGetLastError() != cudaSuccess) rc = 3;
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (out) cudaFree(out);
  cudaGetLastError();
  return rc;
}

extern "C" int sbdgb_measure_fp64_rates(int device, double *dfma_tflops, double *dmma_tflops) {
  if (!dfma_tflops || !dmma_tflops) return 1;
  int sms = 0;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
    cudaGetLastError();
    return 3;
  }
  const int blocks = sms * 8;
  double *out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaStream_t s = nullptr;
  int rc = 0;
  if (cudaMalloc(&out, sizeof(double) * blocks) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
      cudaEventCreate(&e1) != cudaSuccess || cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
    rc = 3;
  float ms_fma = 0.f, ms_mma = 0.f;
  for (int rep = 0; rep < 2 && rc == 0; ++rep) {  // the first run is untimed
    cudaEventRecord(e0, s);
    k_rate_dfma<<<blocks, kRateThreads, 0, s>>>(out);
    cudaEventRecord(e1, s);
    if (cudaEventSynchronize(e1) != cudaSuccess) rc = 3;
    cudaEventElapsedTime(&ms_fma, e0, e1);
    cudaEventRecord(e0, s);
    k_rate_dmma<<<blocks, kRateThreads, 0, s>>>(out);
    cudaEventRecord(e1, s);
    if (cudaEventSynchronize(e1) != cudaSuccess) rc = 3;
    cudaEventElapsedTime(&ms_mma, e0, e1);
  }
  if (rc == 0 && cudaGetLastError() != cudaSuccess) rc = 3;
  if (rc == 0) {
    // FMAs: 8 per thread per iteration; one m8n8k4 per warp is 256 FMAs, 4 per iteration
    const double fma = (double)blocks * kRateThreads * kRateIters * 8;
    const double mma = (double)blocks * (kRateThreads / 32) * kRateIters * 4 * 256;
    *dfma_tflops = 2.0 * fma / (ms_fma * 1e-3) / 1e12;
    *dmma_tflops = 2.0 * mma / (ms_mma * 1e-3) / 1e12;
  }
  if (s) cudaStreamDestroy(s);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (out) cudaFree(out);
  cudaGetLastError();
  return rc;
}
