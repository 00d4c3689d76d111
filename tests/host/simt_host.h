// simt_host.h - runs CUDA device code of this repository on the host, for
// the CPU test suite.  TEST INFRASTRUCTURE ONLY.
//
// One CTA of `nt` threads is `nt` std::threads.  threadIdx is thread-local,
// __syncthreads is a barrier of the CTA, a warp shuffle is an exchange
// through a per-warp slot array between two barriers of the warp (every
// shuffle of this code is executed by full warps), and __shared__ data is
// the caller's.  The SIMD integer intrinsics the DP uses are written here
// from their documented per-lane meaning: 16-bit lanes add with wrap-around,
// maxima compare lanes as signed values.
#pragma once

#include <algorithm>
#include <atomic>
#include <barrier>
#include <cstdint>
#include <cstring>
#include <functional>
#include <memory>
#include <optional>
#include <thread>
#include <vector>
#ifdef SIMT_TRACE
#include <atomic>
#include <cstdio>
#endif

#define SPOA_GB300_SIMT_HOST 1
#define __host__
#define __device__
#define __forceinline__ inline
#define __noinline__

struct uint2 {
  unsigned int x, y;
};
struct int4 {
  int x, y, z, w;
};
struct uint4 {
  unsigned int x, y, z, w;
};
static inline uint2 make_uint2(unsigned a, unsigned b) { return uint2{a, b}; }
static inline int4 make_int4(int a, int b, int c, int d) { return int4{a, b, c, d}; }
static inline uint4 make_uint4(unsigned a, unsigned b, unsigned c, unsigned d) {
  return uint4{a, b, c, d};
}
using std::max;
using std::min;

struct HostDim {
  unsigned x;
};

namespace simt {

// One CTA, or a cluster of `ncta` CTAs of `nt` threads each (the threads of
// CTA r are ranks r * nt ... r * nt + nt - 1 of the launch).
struct Cta {
  unsigned nt = 1, ncta = 1;
  std::vector<std::unique_ptr<std::barrier<>>> cta_bar;  // per CTA
  std::unique_ptr<std::barrier<>> cluster_bar;           // all threads
  std::vector<std::unique_ptr<std::barrier<>>> warp;     // per CTA and warp
  std::vector<int32_t> slots;                            // 32 per warp
  std::vector<char*> scratch;  // per CTA: its shared-memory stand-in
};

inline Cta*& cta() {
  static Cta* c = nullptr;
  return c;
}
inline thread_local HostDim tid{0};
inline thread_local unsigned cta_rank = 0;

// Runs body() on ncta CTAs of nt threads (a cluster when ncta > 1);
// scratch[r] is CTA r's shared-memory stand-in (for the distributed shared
// memory of a cluster).  Returns when all threads have finished.
inline void launch_cluster(unsigned ncta, unsigned nt, const std::vector<char*>& scratch,
                           const std::function<void()>& body) {
  Cta c;
  c.nt = nt;
  c.ncta = ncta;
  c.scratch = scratch;
  for (unsigned r = 0; r < ncta; ++r) c.cta_bar.push_back(std::make_unique<std::barrier<>>(nt));
  c.cluster_bar = std::make_unique<std::barrier<>>(nt * ncta);
  const unsigned nw = (nt + 31) / 32;
  for (unsigned r = 0; r < ncta; ++r)
    for (unsigned w = 0; w < nw; ++w)
      c.warp.push_back(std::make_unique<std::barrier<>>(std::min(32u, nt - 32 * w)));
  c.slots.assign(32 * nw * ncta, 0);
  cta() = &c;
  std::vector<std::thread> th;
  for (unsigned r = 0; r < ncta; ++r)
    for (unsigned t = 0; t < nt; ++t)
      th.emplace_back([r, t, &body] {
        tid.x = t;
        cta_rank = r;
        body();
      });
  for (auto& x : th) x.join();
  cta() = nullptr;
}

// Runs body() on nt threads as one CTA; returns when all have finished.
inline void launch(unsigned nt, const std::function<void()>& body) {
  launch_cluster(1, nt, {}, body);
}

inline int32_t exchange(int32_t v, unsigned src_lane) {
  Cta& c = *cta();
  const unsigned w = cta_rank * ((c.nt + 31) / 32) + tid.x / 32, lane = tid.x % 32;
  c.slots[32 * w + lane] = v;
  c.warp[w]->arrive_and_wait();
  const int32_t r = c.slots[32 * w + src_lane];
  c.warp[w]->arrive_and_wait();
  return r;
}

inline void cluster_sync() {
  if (cta()) cta()->cluster_bar->arrive_and_wait();
}

// The split form: arrive, then (after other work) wait for the others.
inline thread_local std::optional<std::barrier<>::arrival_token> cluster_token;
inline void cluster_arrive() {
  if (cta()) cluster_token.emplace(cta()->cluster_bar->arrive());
}
inline void cluster_wait() {
  if (cta() && cluster_token) {
    cta()->cluster_bar->wait(std::move(*cluster_token));
    cluster_token.reset();
  }
}

// The copy of a shared variable of this CTA in CTA `rank` of the cluster.
template <typename T>
inline T* peer(T* local, unsigned rank) {
  Cta& c = *cta();
  const std::ptrdiff_t off = reinterpret_cast<const char*>(local) - c.scratch[cta_rank];
  return reinterpret_cast<T*>(c.scratch[rank] + off);
}

}  // namespace simt

#define threadIdx (simt::tid)
static struct BlockDimProxy {
  struct X {
    operator unsigned() const { return simt::cta() ? simt::cta()->nt : 1u; }
  } x;
} blockDim;
static const HostDim blockIdx{0};

static inline void __syncthreads() {
#ifdef SIMT_TRACE
  static std::atomic<long> n{0};
  if (threadIdx.x == 0) fprintf(stderr, "sync %ld\n", n++);
#endif
  if (simt::cta()) simt::cta()->cta_bar[simt::cta_rank]->arrive_and_wait();
}

template <typename T>
static inline T __shfl_up_sync(unsigned, T v, unsigned d) {
  const unsigned lane = threadIdx.x % 32;
  int32_t bits;
  std::memcpy(&bits, &v, sizeof(bits));
  const int32_t r = simt::exchange(bits, lane >= d ? lane - d : lane);
  T out;
  std::memcpy(&out, &r, sizeof(out));
  return out;
}

template <typename T>
static inline T __shfl_xor_sync(unsigned, T v, unsigned m) {
  const unsigned lane = threadIdx.x % 32;
  int32_t bits;
  std::memcpy(&bits, &v, sizeof(bits));
  const int32_t r = simt::exchange(bits, (lane ^ m) % 32);
  T out;
  std::memcpy(&out, &r, sizeof(out));
  return out;
}

template <typename T>
static inline T __shfl_sync(unsigned, T v, int src) {
  int32_t bits;
  std::memcpy(&bits, &v, sizeof(bits));
  const int32_t r = simt::exchange(bits, (unsigned)src % 32);
  T out;
  std::memcpy(&out, &r, sizeof(out));
  return out;
}

static inline unsigned __ballot_sync(unsigned, int pred) {
  unsigned m = 0;
  for (unsigned l = 0; l < 32; ++l) m |= (unsigned)(simt::exchange(pred ? 1 : 0, l) != 0) << l;
  return m;
}

static inline int __ffs(unsigned x) { return x ? __builtin_ctz(x) + 1 : 0; }

static inline void __syncwarp(unsigned = 0xffffffffu) {
  if (simt::cta()) {
    simt::Cta& c = *simt::cta();
    c.warp[simt::cta_rank * ((c.nt + 31) / 32) + threadIdx.x / 32]->arrive_and_wait();
  }
}

// ---- SIMD integer intrinsics, per their documented lane semantics ----
namespace simt {
inline int32_t lo16(uint32_t x) { return (int16_t)(x & 0xFFFFu); }
inline int32_t hi16(uint32_t x) { return (int16_t)(x >> 16); }
inline uint32_t pack16(int32_t lo, int32_t hi) {
  return ((uint32_t)(uint16_t)lo) | ((uint32_t)(uint16_t)hi << 16);
}
}  // namespace simt

static inline uint32_t __vadd2(uint32_t a, uint32_t b) {
  return simt::pack16(simt::lo16(a) + simt::lo16(b), simt::hi16(a) + simt::hi16(b));
}
static inline uint32_t __vimax3_s16x2(uint32_t a, uint32_t b, uint32_t c) {
  using namespace simt;
  return pack16(std::max({lo16(a), lo16(b), lo16(c)}), std::max({hi16(a), hi16(b), hi16(c)}));
}
static inline uint32_t __vimax3_s16x2_relu(uint32_t a, uint32_t b, uint32_t c) {
  using namespace simt;
  return pack16(std::max({lo16(a), lo16(b), lo16(c), 0}), std::max({hi16(a), hi16(b), hi16(c), 0}));
}
static inline uint32_t __viaddmax_s16x2(uint32_t a, uint32_t b, uint32_t c) {
  using namespace simt;
  const uint32_t s = __vadd2(a, b);  // the sum wraps in its 16-bit lane
  return pack16(std::max(lo16(s), lo16(c)), std::max(hi16(s), hi16(c)));
}
static inline int32_t __vimax3_s32(int32_t a, int32_t b, int32_t c) { return std::max({a, b, c}); }
static inline int32_t __vimax3_s32_relu(int32_t a, int32_t b, int32_t c) {
  return std::max({a, b, c, 0});
}
static inline int32_t __viaddmax_s32(int32_t a, int32_t b, int32_t c) {
  return std::max((int32_t)((uint32_t)a + (uint32_t)b), c);
}
// byte s[4k+3:4k] of the selector picks byte n of the 8 bytes {y, x}
static inline uint32_t __byte_perm(uint32_t x, uint32_t y, uint32_t s) {
  const uint64_t v = ((uint64_t)y << 32) | x;
  uint32_t r = 0;
  for (int k = 0; k < 4; ++k) r |= (uint32_t)((v >> (8 * ((s >> (4 * k)) & 7))) & 0xFF) << (8 * k);
  return r;
}
template <typename T>
static inline void __stcs(T* p, T v) {
  *p = v;
}
static inline uint32_t atomicAdd(uint32_t* p, uint32_t v) {
  return std::atomic_ref<uint32_t>(*p).fetch_add(v);
}
static inline unsigned long long atomicAdd(unsigned long long* p, unsigned long long v) {
  return std::atomic_ref<unsigned long long>(*p).fetch_add(v);
}
