// int_peak.cu - measures the sustained rate of the integer max/add
// instructions the DP runs on, for the integer roofline of the benchmark:
// the 32-bit forms (__viaddmax_s32, __vimax3_s32, int32 add) of the 32-bit
// kernels and the 16x2 forms (__viaddmax_s16x2, __vimax3_s16x2, __vadd2,
// two DP cells per instruction) of the 16-bit kernels.  Not part of the C
// ABI.
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

// The same chains on int16x2 pairs; the penalties come from the seed so the
// compiler cannot fold them.
__global__ void __launch_bounds__(256) k_int_peak16(int32_t* out, int32_t iters, int32_t seed) {
  uint32_t a[kChains], b[kChains];
  const uint32_t p3 = 0xFFFDFFFDu + (uint32_t)(seed >> 20);  // -3 in both lanes
  const uint32_t p5 = 0xFFFBFFFBu + (uint32_t)(seed >> 21);
  const uint32_t p7 = 0xFFF9FFF9u + (uint32_t)(seed >> 22);
#pragma unroll
  for (int k = 0; k < kChains; ++k) {
    a[k] = (uint32_t)(seed + threadIdx.x + k) * 0x00010001u;
    b[k] = (uint32_t)(seed - k) * 0x00010001u;
  }
  for (int32_t it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < kChains; ++k) {
      a[k] = __viaddmax_s16x2(a[k], p3, b[k]);
      b[k] = __vimax3_s16x2(__vadd2(b[k], p5), a[k], __vadd2(b[k], p7));
    }
  }
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += a[k] ^ b[k];
  if (s == 0x7fffffffu) out[0] = (int32_t)s;
}

template <typename K>
double time_probe(K kernel, int32_t iters, double ops_per_step) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int32_t* out = nullptr;
  if (cudaMalloc(&out, 4) != cudaSuccess) return -1;
  const int threads = 256, blocks = sms * 8;
  kernel<<<blocks, threads>>>(out, 16, 1);  // warm-up
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 0;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    kernel<<<blocks, threads>>>(out, iters, 2 + rep);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep == 0 || ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (cudaGetLastError() != cudaSuccess || best <= 0) return -1;
  const double ops = (double)blocks * threads * kChains * iters * ops_per_step;
  return ops / (best * 1e-3);
}

}  // namespace

// Integer lane-operations per second of the 32-bit forms, counting each
// __viaddmax_s32, each __vimax3_s32 and each int32 add as one operation
// (the unit in which the DP's per-cell operation counts are stated), or a
// negative value on error.  Per chain step: one viaddmax, two adds, one
// vimax3.
extern "C" double spoa_gb300_int_peak_ops(int32_t iters) {
  return time_probe(k_int_peak, iters, 4.0);
}

// The same for the 16x2 forms the 16-bit kernels issue: each
// __viaddmax_s16x2, __vimax3_s16x2 and __vadd2 is two lane-operations (one
// per DP cell).  Per chain step: one viaddmax, two vadd2, one vimax3.
extern "C" double spoa_gb300_int_peak_ops16x2(int32_t iters) {
  return time_probe(k_int_peak16, iters, 8.0);
}
