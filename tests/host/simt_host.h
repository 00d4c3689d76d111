// simt_host.h - runs CUDA device code of this repository on the host, for
// the CPU test suite.  TEST INFRASTRUCTURE ONLY.
//
// One CTA of `nt` threads is `nt` fibers (ucontext) on the calling OS
// thread.  A fiber runs until it waits at a barrier; threadIdx is set for
// the fiber that runs.  __syncthreads is a barrier of the CTA, a warp
// shuffle is an exchange through per-warp slot arrays behind one barrier of
// the warp (every shuffle of this code is executed by full warps), and
// __shared__ data is the caller's.  A barrier that can never complete
// aborts the launch with the place each thread waits, and so do threads
// that meet at two different calls of an aligned barrier (__syncthreads,
// the cluster barrier).  The SIMD integer intrinsics the DP uses are
// written here from their documented per-lane meaning: 16-bit lanes add
// with wrap-around, maxima compare lanes as signed values.
#pragma once

#include <sys/mman.h>
#include <ucontext.h>

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <functional>
#include <source_location>
#include <vector>

// Built with -fsanitize=thread, the emulation is a race detector for the
// device code: fibers switch without ordering each other, and the only
// happens-before edges are the ones a GPU gives (barrier arrive -> barrier
// completion, launch -> threads -> launch end, atomics), so two threads that
// touch the same shared or global bytes between barriers, one of them
// writing, are reported with both stacks.
#if defined(__SANITIZE_THREAD__)
#include <sanitizer/tsan_interface.h>
#define SIMT_RACECHECK 1
extern "C" void AnnotateIgnoreReadsBegin(const char* file, int line);
extern "C" void AnnotateIgnoreReadsEnd(const char* file, int line);
extern "C" void AnnotateIgnoreWritesBegin(const char* file, int line);
extern "C" void AnnotateIgnoreWritesEnd(const char* file, int line);
#endif

// Built with -fsanitize=address, the fiber switches are announced to
// AddressSanitizer (the stack each switch lands on), so that it keeps
// checking the emulated threads' stacks; with SPOA_GB300_HOST_REDZONE the
// device arenas of the code under test carry poisoned red zones between
// their regions (poa_device.cuh), so an access past a region is reported.
#if defined(__SANITIZE_ADDRESS__)
#include <pthread.h>
#include <sanitizer/common_interface_defs.h>
#define SIMT_ASAN 1
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

using Site = std::source_location;

// An emulated thread: a fiber with its own stack on the calling OS thread.
struct Fiber {
  ucontext_t ctx;
  unsigned t = 0, r = 0;  // threadIdx.x and CTA rank
  bool done = false;
  bool has_token = false;  // between cluster_arrive and cluster_wait
  uint64_t token = 0;      // the cluster barrier's phase at the arrive
  const char* waits_on = nullptr;  // kind of barrier it is blocked on
  uint64_t shuffles = 0;           // warp shuffles done (picks the slot array)
  void* race_ctx = nullptr;        // the race detector's fiber (racecheck builds)
  void* asan_fake = nullptr;       // AddressSanitizer's state of this stack
};

// A barrier of `expected` fibers; `phase` counts completed rounds.
struct Barrier {
  unsigned expected = 0, arrived = 0;
  uint64_t phase = 0;
  std::vector<unsigned> waiting;  // fibers blocked on the current phase
  char order[2] = {0, 0};  // happens-before keys of even and odd phases (racecheck)
  const char* site_file = nullptr;  // where the current phase's first thread
  unsigned site_line = 0;           // called the barrier (aligned barriers)
};

// One CTA, or a cluster of `ncta` CTAs of `nt` threads each (the threads of
// CTA r are fibers r * nt ... r * nt + nt - 1 of the launch).
struct Cta {
  unsigned nt = 1, ncta = 1;
  std::vector<Barrier> cta_bar;  // per CTA
  Barrier cluster_bar;           // all threads
  std::vector<Barrier> warp;     // per CTA and warp
  std::vector<int32_t> slots;    // 2 x 32 per warp (alternating shuffles)
  std::vector<char*> scratch;    // per CTA: its shared-memory stand-in
  std::vector<Fiber> fib;
  std::deque<unsigned> runq;  // fibers ready to run, in order
  unsigned cur = 0;           // the running fiber
  ucontext_t sched;           // the launching code's context
  const std::function<void()>* body = nullptr;
  void* race_sched = nullptr;  // the launching code's race-detector context
  const void* sched_stack = nullptr;  // the launching thread's stack (AddressSanitizer)
  size_t sched_stack_size = 0;
  void* sched_asan_fake = nullptr;
  char order_start = 0, order_end = 0;  // launch -> threads -> launch end
};

inline Cta*& cta() {
  static Cta* c = nullptr;
  return c;
}
inline thread_local HostDim tid{0};
inline thread_local unsigned cta_rank = 0;

// Fiber stacks, kept for the process's lifetime and reused by every launch;
// the lowest page of each is a guard page, so an overflow faults instead of
// overwriting a neighbour.
#ifdef SIMT_ASAN
// AddressSanitizer clears the shadow of the stack a switch lands on, so
// its builds keep the stacks small
constexpr size_t kStackBytes = 128u << 10;
#else
constexpr size_t kStackBytes = 1u << 20;
#endif
inline std::vector<char*>& stack_pool() {
  static std::vector<char*> pool;
  return pool;
}
inline char* stack_at(size_t k) {
  auto& pool = stack_pool();
  while (pool.size() <= k) {
    void* p = mmap(nullptr, kStackBytes, PROT_READ | PROT_WRITE,
                   MAP_PRIVATE | MAP_ANONYMOUS | MAP_NORESERVE, -1, 0);
    if (p == MAP_FAILED) {
      std::fprintf(stderr, "simt: no memory for a fiber stack\n");
      std::abort();
    }
    mprotect(p, 4096, PROT_NONE);
    pool.push_back(static_cast<char*>(p));
  }
  return pool[k];
}

// The emulator's own bookkeeping (run queue, barrier counters, shuffle
// slots, threadIdx): kept out of the race detector's view for the scope of
// one of these, since it stands for hardware state, not device-code data.
struct Internal {
#ifdef SIMT_RACECHECK
  Internal() {
    AnnotateIgnoreReadsBegin(__FILE__, __LINE__);
    AnnotateIgnoreWritesBegin(__FILE__, __LINE__);
  }
  ~Internal() {
    AnnotateIgnoreWritesEnd(__FILE__, __LINE__);
    AnnotateIgnoreReadsEnd(__FILE__, __LINE__);
  }
#endif
};

// Happens-before edges for the race detector (no-ops in other builds).
inline void order_release(void* key) {
#ifdef SIMT_RACECHECK
  __tsan_release(key);
#else
  (void)key;
#endif
}
inline void order_acquire(void* key) {
#ifdef SIMT_RACECHECK
  __tsan_acquire(key);
#else
  (void)key;
#endif
}
// Tells the race detector which fiber runs next, without ordering the two.
// A macro, and the functions that use it are not instrumented: the
// detector keeps a call stack per fiber, so no instrumented function may
// return between this and the switch of stacks that follows it.
#ifdef SIMT_RACECHECK
#define SIMT_RACE_SWITCH(ctx) __tsan_switch_to_fiber((ctx), __tsan_switch_to_fiber_no_sync)
#define SIMT_SWITCHES __attribute__((no_sanitize_thread))
#elif defined(SIMT_ASAN)
#define SIMT_RACE_SWITCH(ctx) ((void)(ctx))
#define SIMT_SWITCHES __attribute__((no_sanitize_address))
#else
#define SIMT_RACE_SWITCH(ctx) ((void)(ctx))
#define SIMT_SWITCHES
#endif

// AddressSanitizer's view of a switch: before it, the stack it lands on
// (fake = nullptr when the leaving fiber ends); after landing, done.
inline void asan_leave(void** fake, const void* bottom, size_t size) {
#ifdef SIMT_ASAN
  __sanitizer_start_switch_fiber(fake, bottom, size);
#else
  (void)fake, (void)bottom, (void)size;
#endif
}
inline void asan_landed(void* fake) {
#ifdef SIMT_ASAN
  __sanitizer_finish_switch_fiber(fake, nullptr, nullptr);
#else
  (void)fake;
#endif
}

// The race detector's context for fiber k, like the stacks kept and reused
// by every launch (a destroyed detector fiber whose stack is reused did not
// survive the next launch).
inline void* race_ctx_at(size_t k) {
#ifdef SIMT_RACECHECK
  static std::vector<void*> pool;
  while (pool.size() <= k) pool.push_back(__tsan_create_fiber(0));
  return pool[k];
#else
  (void)k;
  return nullptr;
#endif
}

SIMT_SWITCHES inline void fiber_entry() {
  Cta& c = *cta();
  asan_landed(nullptr);
  order_acquire(&c.order_start);
  (*c.body)();
  order_release(&c.order_end);
  {
    Internal in;  // ends before the switch: it counts in this fiber's detector state
    c.fib[c.cur].done = true;
  }
  SIMT_RACE_SWITCH(c.race_sched);
  asan_leave(nullptr, c.sched_stack, c.sched_stack_size);
}  // returns to c.sched through uc_link

// The running fiber waits: the OS thread switches straight to the next
// ready fiber (or back to the scheduler when none is ready); the fiber
// resumes once a barrier release has queued it again.
SIMT_SWITCHES inline void block(const char* kind) {
  Internal in;
  Cta& c = *cta();
  const unsigned me = c.cur;
  c.fib[me].waits_on = kind;
  if (c.runq.empty()) {
    SIMT_RACE_SWITCH(c.race_sched);
    asan_leave(&c.fib[me].asan_fake, c.sched_stack, c.sched_stack_size);
    swapcontext(&c.fib[me].ctx, &c.sched);
  } else {
    const unsigned nx = c.runq.front();
    c.runq.pop_front();
    c.cur = nx;
    c.fib[nx].waits_on = nullptr;
    tid.x = c.fib[nx].t;
    cta_rank = c.fib[nx].r;
    SIMT_RACE_SWITCH(c.fib[nx].race_ctx);
    asan_leave(&c.fib[me].asan_fake, stack_at(nx) + 4096, kStackBytes - 4096);
    swapcontext(&c.fib[me].ctx, &c.fib[nx].ctx);
  }
  // resumed: whoever switched here set c.cur, tid and cta_rank to this fiber
  asan_landed(c.fib[me].asan_fake);
}

// Arrives at `b`; the last arrival of a phase releases the waiting fibers.
// Released fibers are queued in arrival order on even phases and in reverse
// order on odd ones, so that code between two barriers runs in both thread
// orders over a launch (a missing barrier shows in one of them).
inline uint64_t arrive(Barrier& b) {
  Internal in;
  Cta& c = *cta();
  const uint64_t ph = b.phase;
  order_release(&b.order[ph & 1]);
  if (++b.arrived == b.expected) {
    b.arrived = 0;
    ++b.phase;
    if (ph & 1)
      c.runq.insert(c.runq.end(), b.waiting.rbegin(), b.waiting.rend());
    else
      c.runq.insert(c.runq.end(), b.waiting.begin(), b.waiting.end());
    b.waiting.clear();
  }
  return ph;
}

// Waits until the phase that began as `ph` has completed.  The keys of
// even and odd phases alternate: a thread can release phase ph + 2 only
// after every thread has arrived at ph + 1, that is after every thread has
// acquired ph.
inline void wait(Barrier& b, uint64_t ph, const char* kind) {
  Internal in;
  Cta& c = *cta();
  while (b.phase == ph) {
    b.waiting.push_back(c.cur);
    block(kind);
  }
  order_acquire(&b.order[ph & 1]);
}

inline void arrive_and_wait(Barrier& b, const char* kind) { wait(b, arrive(b), kind); }

// Aligned barriers (__syncthreads, the cluster barrier): every thread must
// arrive through the same call in each phase; the first arrival of a phase
// records its place, and a thread arriving from another place aborts the
// launch with both.
inline void check_site(Barrier& b, const Site& site, const char* kind) {
  Internal in;
  if (b.arrived == 0) {
    b.site_file = site.file_name();
    b.site_line = site.line();
  } else if (b.site_line != site.line() || std::strcmp(b.site_file, site.file_name()) != 0) {
    std::fprintf(stderr, "simt: threads of CTA %u meet at different %s barriers: %s:%u and %s:%u\n",
                 cta_rank, kind, b.site_file, b.site_line, site.file_name(),
                 (unsigned)site.line());
    std::abort();
  }
}

// Runs body() on ncta CTAs of nt threads (a cluster when ncta > 1) as
// fibers on the calling OS thread, each running until it waits at a barrier
// (no preemption between barriers); scratch[r] is CTA r's shared-memory
// stand-in (for the distributed shared memory of a cluster).  Returns when
// all threads have finished.  If every unfinished thread waits at a barrier
// that can no longer complete (a barrier one path of the code skips), the
// launch reports where each thread waits and aborts the process instead of
// hanging.
inline void launch_cluster(unsigned ncta, unsigned nt, const std::vector<char*>& scratch,
                           const std::function<void()>& body) {
  Internal in;
  Cta c;
  c.nt = nt;
  c.ncta = ncta;
  c.scratch = scratch;
  c.body = &body;
  c.cta_bar.resize(ncta);
  for (auto& b : c.cta_bar) b.expected = nt;
  c.cluster_bar.expected = nt * ncta;
  const unsigned nw = (nt + 31) / 32;
  c.warp.resize(ncta * nw);
  for (unsigned r = 0; r < ncta; ++r)
    for (unsigned w = 0; w < nw; ++w) c.warp[r * nw + w].expected = std::min(32u, nt - 32 * w);
  c.slots.assign(2 * 32 * nw * ncta, 0);
  const unsigned n = ncta * nt;
  c.fib.resize(n);
  Cta* outer = cta();
  cta() = &c;
  for (unsigned k = 0; k < n; ++k) {
    Fiber& f = c.fib[k];
    f.r = k / nt;
    f.t = k % nt;
    getcontext(&f.ctx);
    f.ctx.uc_stack.ss_sp = stack_at(k) + 4096;
    f.ctx.uc_stack.ss_size = kStackBytes - 4096;
    f.ctx.uc_link = &c.sched;
    makecontext(&f.ctx, fiber_entry, 0);
    f.race_ctx = race_ctx_at(k);
    c.runq.push_back(k);
  }
#ifdef SIMT_RACECHECK
  c.race_sched = __tsan_get_current_fiber();
#endif
#ifdef SIMT_ASAN
  {
    pthread_attr_t at;
    void* addr = nullptr;
    size_t size = 0;
    if (pthread_getattr_np(pthread_self(), &at) == 0) {
      pthread_attr_getstack(&at, &addr, &size);
      pthread_attr_destroy(&at);
    }
    c.sched_stack = addr;
    c.sched_stack_size = size;
  }
#endif
  order_release(&c.order_start);
  const HostDim tid0 = tid;
  const unsigned rank0 = cta_rank;
  while (!c.runq.empty()) {
    c.cur = c.runq.front();
    c.runq.pop_front();
    Fiber& f = c.fib[c.cur];
    f.waits_on = nullptr;
    tid.x = f.t;
    cta_rank = f.r;
    SIMT_RACE_SWITCH(f.race_ctx);
    asan_leave(&c.sched_asan_fake, stack_at(c.cur) + 4096, kStackBytes - 4096);
    swapcontext(&c.sched, &f.ctx);
    asan_landed(c.sched_asan_fake);
  }
  for (const Fiber& f : c.fib)
    if (!f.done) {
      std::fprintf(stderr, "simt: barrier deadlock (%u CTAs of %u threads):\n", ncta, nt);
      for (const Fiber& g : c.fib)
        if (!g.done)
          std::fprintf(stderr, "  CTA %u thread %u waits at a %s barrier\n", g.r, g.t,
                       g.waits_on ? g.waits_on : "?");
      std::abort();
    }
  order_acquire(&c.order_end);
  tid = tid0;
  cta_rank = rank0;
  cta() = outer;
}

// Runs body() on nt threads as one CTA; returns when all have finished.
inline void launch(unsigned nt, const std::function<void()>& body) {
  launch_cluster(1, nt, {}, body);
}

// A warp shuffle: every lane writes its value, waits for the warp, reads
// the source lane's.  Two slot arrays alternate between shuffles, so one
// warp barrier suffices: a lane can write the array again only after the
// next shuffle's barrier, which every lane reaches after its read.
inline int32_t exchange(int32_t v, unsigned src_lane) {
  Internal in;
  Cta& c = *cta();
  const unsigned nw = c.ncta * ((c.nt + 31) / 32);
  const unsigned w = cta_rank * ((c.nt + 31) / 32) + tid.x / 32, lane = tid.x % 32;
  Fiber& f = c.fib[c.cur];
  int32_t* slots = c.slots.data() + 32 * (w + nw * (f.shuffles++ & 1));
  slots[lane] = v;
  arrive_and_wait(c.warp[w], "warp");
  return slots[src_lane];
}

inline void cluster_sync(const Site& site = Site::current()) {
  if (!cta()) return;
  check_site(cta()->cluster_bar, site, "cluster");
  arrive_and_wait(cta()->cluster_bar, "cluster");
}

// The split form: arrive, then (after other work) wait for the others.
inline void cluster_arrive(const Site& site = Site::current()) {
  if (!cta()) return;
  check_site(cta()->cluster_bar, site, "cluster");
  Internal in;
  Fiber& f = cta()->fib[cta()->cur];
  f.token = arrive(cta()->cluster_bar);
  f.has_token = true;
}
inline void cluster_wait() {
  Internal in;
  if (!cta()) return;
  Fiber& f = cta()->fib[cta()->cur];
  if (!f.has_token) return;
  f.has_token = false;
  wait(cta()->cluster_bar, f.token, "cluster");
}

// The copy of a shared variable of this CTA in CTA `rank` of the cluster.
template <typename T>
inline T* peer(T* local, unsigned rank) {
  Internal in;
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

// __syncthreads is an aligned barrier: every thread of the CTA must reach
// the same one (the same call in the source) in each phase, or the GPU's
// behaviour is undefined.  The emulation checks that and aborts with both
// places when two threads of a CTA meet at different __syncthreads.
static inline void __syncthreads(const simt::Site site = simt::Site::current()) {
#ifdef SIMT_TRACE
  static std::atomic<long> n{0};
  if (threadIdx.x == 0) fprintf(stderr, "sync %ld\n", n++);
#endif
  if (!simt::cta()) return;
  simt::Barrier& b = simt::cta()->cta_bar[simt::cta_rank];
  simt::check_site(b, site, "__syncthreads");
  simt::arrive_and_wait(b, "CTA");
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
    simt::arrive_and_wait(c.warp[simt::cta_rank * ((c.nt + 31) / 32) + threadIdx.x / 32], "warp");
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
