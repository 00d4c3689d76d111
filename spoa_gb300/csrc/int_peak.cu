// int_peak.cu - measures the sustained rate of the integer max/add
// instructions the DP runs on (__viaddmax_s32, __vimax3_s32, int32 add),
// for the integer roofline of the benchmark.  Not part of the C ABI.
//
// Every thread runs independent dependency chains so the pipes, not the
// latency, set the rate; the result is written so nothing is optimised away.
#include <cuda_runtime.h>

#include <cstdint>

namespace {

constexpr int kChains = 8;

__global__ void __launch_bounds__(256) k_int_peak(int32_t* out, int32_t iters, int32_t seed) {
  int32_t a[kChains], b[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) {
    a[k] = seed + threadIdx.x + k;
    b[k] = seed - k;
  }
  for (int32_t it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < kChains; ++k) {
      a[k] = __viaddmax_s32(a[k], -3, b[k]);  // max(a - 3, b)
      b[k] = __vimax3_s32(b[k] - 5, a[k], b[k] - 7);
    }
  }
  int32_t s = 0;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += a[k] ^ b[k];
  if (s == 0x7fffffff) out[0] = s;
}

}  // namespace

// Returns integer lane-operations per second, counting each __viaddmax_s32,
// each __vimax3_s32 and each int32 add as one operation (the unit in which
// the DP's per-cell operation counts are stated), or a negative value on
// error.
extern "C" double spoa_gb300_int_peak_ops(int32_t iters) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int32_t* out = nullptr;
  if (cudaMalloc(&out, 4) != cudaSuccess) return -1;
  const int threads = 256, blocks = sms * 8;
  k_int_peak<<<blocks, threads>>>(out, 16, 1);  // warm-up
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0);
  k_int_peak<<<blocks, threads>>>(out, iters, 2);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (cudaGetLastError() != cudaSuccess || ms <= 0) return -1;
  // per chain step: one viaddmax, two adds, one vimax3
  const double ops = (double)blocks * threads * kChains * iters * 4.0;
  return ops / (ms * 1e-3);
}
