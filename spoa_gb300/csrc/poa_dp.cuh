// poa_dp.cuh - graph-to-sequence DP of one read against one window's graph,
// run by one CTA, and its traceback.
//
// Layout: row i (1-based rank + 1, row 0 is the initial row) x column j
// (read position).  Thread t owns the strip of CPT consecutive columns
// [t*CPT, (t+1)*CPT), held as CPT/2 lane pairs (column s+k with column
// s+CPT/2+k) so one int16x2 DPX instruction advances both half-strips.
// Rows are processed in rank order; the previous row stays in registers and
// other predecessor rows are read back from the H/F/O rows in HBM (they can
// be any earlier row).  The in-row gap recurrences are max-plus linear scans
//     X[j] = max(a[j], X[j-1] + pen)
// computed as a per-thread strip scan, a CTA-wide exclusive prefix-max of
// the strip aggregates (warp shuffles + shared memory) and a fix-up pass.
//
// Semantics follow the AVX2 SimdAlignmentEngine cell by cell
// (src/simd_alignment_engine_implementation.hpp):
//   F = max_p(max(H_p + (g-e), F_p) + e)          (1199-1203, 1226-1232)
//   O = max_p(max(H_p + (q-c), O_p) + c)          (1667-1671, 1704-1710)
//   Hd = max_p(H_p[j-1] + profile)                 (1206-1210)
//   H1 = max(Hd, F, O)                             (1734-1736)
//   Q[j] = max(H1[j-1] + q, Q[j-1] + c), Q[0] = fc + q     (1748-1756)
//   E[j] = max(H1[j-1] + g, E[j-1] + e), E[0] = fc + g     (1738-1746)
//          and, in convex mode only, at vector starts (j % lanes == 0)
//          also Q[j-1] + g: the carried lane is the previous vector's
//          final H, which includes Q (1762-1764)
//   H = max(H1, E, Q); SW stores max(H, 0) but E/Q carry the unclamped H
// In the scans the recurrences are shifted by one column (E'[k] = E[k+1])
// so that every input of a strip is owned by the strip's thread.
#pragma once

#include "poa_device.cuh"

namespace spoa_gb300 {

__device__ __forceinline__ int32_t imax(int32_t a, int32_t b) { return a > b ? a : b; }
__device__ __forceinline__ int32_t imax3(int32_t a, int32_t b, int32_t c) {
  return __vimax3_s32(a, b, c);
}
// max(a + b, c) on the DPX path
__device__ __forceinline__ int32_t addmax(int32_t a, int32_t b, int32_t c) {
  return __viaddmax_s32(a, b, c);
}

struct BlockScratch {
  // per-warp slots of the in-row exchanges, one array per exchange of a
  // row (the Q scan, the E / H scan, the left column): the next write to a
  // slot comes after another exchange's barrier, so none needs a barrier
  // after its reads.  wv2 takes the left column during the row loop and
  // the block reductions after it (each of those starts with a barrier).
  int32_t wq[32];
  int32_t wv[32];
  int32_t wv2[32];
  int32_t bcast[8];
  int32_t cl[8];      // values this CTA publishes to the other CTAs of its cluster
  int32_t clx[2][8];  // its row tails (cluster_publish), by row parity
};

// ---------------------------------------------------------------------------
// thread-block clusters: one long window's row spread over CL CTAs
// ---------------------------------------------------------------------------
// CTA r of a cluster of CL owns virtual threads r * nt ... r * nt + nt - 1
// of the row.  What a row carries across CTAs (its scans' tails and the
// left column) crosses in one exchange per row (cluster_publish /
// cluster_fold), the final reductions in one exchange each, all through
// distributed shared memory behind a cluster barrier; every CTA of the
// cluster runs the same sequence of barriers (the control flow is uniform
// over the cluster).
template <int CL>
__device__ __forceinline__ uint32_t cl_rank() {
  if constexpr (CL == 1) {
    return 0;
  } else {
#ifdef __CUDA_ARCH__
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
#elif defined(SPOA_GB300_SIMT_HOST)
    return simt::cta_rank;
#else
    return 0;
#endif
  }
}

// In the host emulation of the device code (tests only), the cluster
// barriers take the place they are called from, so that the emulation can
// check that every thread meets the same (aligned) barrier.
#ifdef SPOA_GB300_SIMT_HOST
#define SPOA_GB300_BARRIER_SITE const simt::Site site = simt::Site::current()
#else
#define SPOA_GB300_BARRIER_SITE
#endif

// Barrier of the whole cluster (of the CTA when CL == 1), ordering the
// memory operations before it against those after it for all its threads.
template <int CL>
__device__ __forceinline__ void cl_sync(SPOA_GB300_BARRIER_SITE) {
  if constexpr (CL == 1) {
#ifdef SPOA_GB300_SIMT_HOST
    __syncthreads(site);
#else
    __syncthreads();
#endif
  } else {
#ifdef __CUDA_ARCH__
    asm volatile("barrier.cluster.arrive.release.aligned;\n\t"
                 "barrier.cluster.wait.acquire.aligned;" ::: "memory");
#elif defined(SPOA_GB300_SIMT_HOST)
    simt::cluster_sync(site);
#endif
  }
}

// The split form of cl_sync (CL > 1): arrive, releasing this thread's
// earlier memory operations to the cluster; other work; then wait for every
// thread of the cluster to arrive, acquiring theirs.  Memory operations
// between the two are not ordered by the barrier.
template <int CL>
__device__ __forceinline__ void cl_arrive(SPOA_GB300_BARRIER_SITE) {
#ifdef __CUDA_ARCH__
  asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
#elif defined(SPOA_GB300_SIMT_HOST)
  simt::cluster_arrive(site);
#endif
}
template <int CL>
__device__ __forceinline__ void cl_wait() {
#ifdef __CUDA_ARCH__
  asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
#elif defined(SPOA_GB300_SIMT_HOST)
  simt::cluster_wait();
#endif
}

// A 32-bit shared variable of CTA `rank` of the cluster (the same variable
// as `local` in this CTA).
__device__ __forceinline__ int32_t cl_peek(const int32_t* local, uint32_t rank) {
#ifdef __CUDA_ARCH__
  const uint32_t sa = (uint32_t)__cvta_generic_to_shared(local);
  uint32_t ra;
  int32_t v;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(sa), "r"(rank));
  asm volatile("ld.shared::cluster.b32 %0, [%1];" : "=r"(v) : "r"(ra) : "memory");
  return v;
#elif defined(SPOA_GB300_SIMT_HOST)
  return *simt::peer(local, rank);
#else  // the host pass of nvcc, which never runs device code
  (void)rank;
  return *local;
#endif
}

// Slots of BlockScratch::cl: the final row maximum, minimum row and minimum
// column.
enum : int { kClMax = 0, kClMin = 1, kClMinJ = 2 };

// Exclusive prefix-max of v over the CTA's threads (kNegBig for thread 0).
// NW: warps of the CTA when known at compile time (0: blockDim.x / 32).
// `slots` (32 per-warp values) must not be written again before the CTA's
// next barrier.
template <int NW = 0>
__device__ __forceinline__ int32_t block_excl_max(int32_t v, int32_t* slots) {
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t nw = NW ? NW : blockDim.x >> 5;
  int32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x = imax(x, y);
  }
  int32_t ex = __shfl_up_sync(0xffffffffu, x, 1);
  if (lane == 0) ex = kNegBig;
  if (nw > 1) {
    if (lane == 31) slots[warp] = x;
    __syncthreads();
    int32_t wp = kNegBig;
    for (uint32_t w = 0; w < warp; ++w) wp = imax(wp, slots[w]);
    ex = imax(ex, wp);
  }
  return ex;
}

template <int NW = 0>
__device__ __forceinline__ int32_t block_max(int32_t v, BlockScratch& sh);
template <int NW = 0>
__device__ __forceinline__ int32_t block_min(int32_t v, BlockScratch& sh);

// The maximum / minimum of v over every thread of the cluster (every
// thread gets it); `slot` is the BlockScratch::cl entry the exchange uses.
template <int NW, int CL>
__device__ __forceinline__ int32_t cluster_max(int32_t v, BlockScratch& sh, int slot) {
  v = block_max<NW>(v, sh);
  if constexpr (CL > 1) {
    if (threadIdx.x == 0) sh.cl[slot] = v;
    cl_sync<CL>();
    for (uint32_t r = 0; r < (uint32_t)CL; ++r) v = imax(v, cl_peek(&sh.cl[slot], r));
  }
  return v;
}
template <int NW, int CL>
__device__ __forceinline__ int32_t cluster_min(int32_t v, BlockScratch& sh, int slot) {
  v = block_min<NW>(v, sh);
  if constexpr (CL > 1) {
    if (threadIdx.x == 0) sh.cl[slot] = v;
    cl_sync<CL>();
    for (uint32_t r = 0; r < (uint32_t)CL; ++r) v = min(v, cl_peek(&sh.cl[slot], r));
  }
  return v;
}

template <int NW>
__device__ __forceinline__ int32_t block_max(int32_t v, BlockScratch& sh) {
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t nw = NW ? NW : blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = imax(v, __shfl_xor_sync(0xffffffffu, v, o));
  if (nw > 1) {
    __syncthreads();
    if (lane == 0) sh.wv2[warp] = v;
    __syncthreads();
    v = kNegBig;
    for (uint32_t w = 0; w < nw; ++w) v = imax(v, sh.wv2[w]);
    __syncthreads();
  }
  return v;
}

template <int NW>
__device__ __forceinline__ int32_t block_min(int32_t v, BlockScratch& sh) {
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t nw = NW ? NW : blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
  if (nw > 1) {
    __syncthreads();
    if (lane == 0) sh.wv2[warp] = v;
    __syncthreads();
    v = 0x7fffffff;
    for (uint32_t w = 0; w < nw; ++w) v = min(v, sh.wv2[w]);
    __syncthreads();
  }
  return v;
}

// Carry X[s-1] into strip t (s = t*CPT) of the scan
//   X[j] = max(a[j], X[j-1] + pen),  X[-1] = init,
// given the strip aggregate agg = max_k a[s+k] + (CPT-1-k)*pen.
//   X[s-1] = max(init + s*pen, max_{t'<t} agg_t' + (t-1-t')*CPT*pen)
// With b_t = agg_t - t*CPT*pen this is a plain prefix-max.  Only thread 0
// knows `init`; it folds it into its own aggregate (its strip end is then
// exactly X[CPT-1]), so the other threads never need it.
template <int CPT, int NW = 0>
__device__ __forceinline__ int32_t scan_carry(int32_t agg, int32_t init, int32_t pen,
                                              int32_t* slots) {
  const int32_t t = (int32_t)threadIdx.x;
  const int32_t D = CPT * pen;
  int32_t v = t == 0 ? imax(agg, init + D) : agg;
  const int32_t x = v - t * D;
  const int32_t ex = block_excl_max<NW>(x, slots);
  return t == 0 ? init : ex + (t - 1) * D;
}

// row flags: sink node; the previous row is a predecessor; source node (row
// 0 is its only predecessor); more than two predecessors besides the
// previous row
constexpr uint8_t kRowSink = 1, kRowPrevPred = 2, kRowSource = 4, kRowMore = 8;

// Builds the rank-ordered predecessor lists of the graph into the DP arena:
// row i = rank + 1; preds of a source row = {0}.
static __device__ __noinline__ void dp_build_rows(const GraphView& G, DpView& D, BlockScratch& sh) {
  const uint32_t V = G.hdr->n_nodes;
  const uint32_t nt = blockDim.x, t = threadIdx.x;
  const uint32_t chunk = (V + nt - 1) / nt;
  const uint32_t r0 = min(V, t * chunk), r1 = min(V, r0 + chunk);
  uint32_t cnt = 0;
  for (uint32_t r = r0; r < r1; ++r) {
    uint32_t d = G.in_deg[G.rank_to_node[r]];
    cnt += d ? d : 1;
  }
  // exclusive sum of cnt over threads
  __syncthreads();
  uint32_t x = cnt;
  const uint32_t lane = t & 31, warp = t >> 5, nw = nt >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  uint32_t ex = x - cnt;
  if (lane == 31) sh.wv[warp] = (int32_t)x;
  __syncthreads();
  for (uint32_t w = 0; w < warp && w < nw; ++w) ex += (uint32_t)sh.wv[w];
  __syncthreads();
  uint32_t off = ex;
  for (uint32_t r = r0; r < r1; ++r) {
    const uint32_t node = G.rank_to_node[r];
    const uint32_t i = r + 1;
    D.pred_ptr[i] = off;
    const uint32_t d = G.in_deg[node];
    D.row_indeg[i] = d;
    const uint8_t ch = (uint8_t)G.hdr->decoder[G.code[node]];
    D.row_char[i] = ch;
    uint8_t flags = G.nlink[node].z == kNone ? kRowSink : 0;
    const uint32_t begin = off;
    uint32_t other[2] = {kNone, kNone}, n_other = 0;
    if (d == 0) {
      D.preds[off++] = 0;
      flags |= kRowSource;
      if (i == 1) flags |= kRowPrevPred;
      else other[n_other++] = 0;
    } else {
      for (uint32_t e = G.nlink[node].x; e != kNone; e = G.erec[e].z) {
        const uint32_t p = G.node_to_rank[G.erec[e].x] + 1;
        D.preds[off++] = p;
        if (p == i - 1) {
          flags |= kRowPrevPred;
        } else {
          if (n_other < 2) other[n_other] = p;
          ++n_other;
        }
      }
    }
    if (n_other > 2) flags |= kRowMore;
    D.row_sink[i] = flags;
    D.rowrec[i] = make_uint4(begin, min(off - begin, 0xFFFFu) | (uint32_t)flags << 16 |
                                        (uint32_t)ch << 24,
                             other[0], other[1]);
  }
  if (t == nt - 1) D.pred_ptr[V + 1] = off;
  __syncthreads();
}

// ---------------------------------------------------------------------------
// lane pairs: two DP columns per operation
// ---------------------------------------------------------------------------
// Lanes<int16_t>: the pair lives in one 32-bit register (int16x2) and every
// max/add is one DPX or SIMD instruction for both columns; used when the
// reference's width rule picks int16 (16 lanes).  Lanes<int32_t>: two
// registers, scalar DPX instructions; used for the int32 width (8 lanes).
// Select masks have the same format in both: 0xFFFF in the low half for the
// first column, 0xFFFF0000 for the second; equality tests (eqb) return bit 15
// for the first column and bit 31 for the second.
template <typename T>
struct Lanes;

template <>
struct Lanes<int16_t> {
  struct P {
    uint32_t v;
  };
  static constexpr int32_t kNeg = INT16_MIN + 1024;
  __device__ __forceinline__ static P make(int32_t lo, int32_t hi) {
    return {(uint32_t)(uint16_t)lo | ((uint32_t)(uint16_t)hi << 16)};
  }
  __device__ __forceinline__ static P splat(int32_t x) { return make(x, x); }
  __device__ __forceinline__ static int32_t lo(P a) { return (int32_t)(int16_t)(a.v & 0xFFFFu); }
  __device__ __forceinline__ static int32_t hi(P a) { return (int32_t)(int16_t)(a.v >> 16); }
  __device__ __forceinline__ static P add(P a, P b) { return {__vadd2(a.v, b.v)}; }
  // max(a, b) as one DPX instruction; nz must be INT16_MIN in both lanes,
  // held in a register (Scoring::min16x2)
  __device__ __forceinline__ static P max(P a, P b, uint32_t nz) {
    return {__vimax3_s16x2(a.v, b.v, nz)};
  }
  // max(a, b, c, 0)
  __device__ __forceinline__ static P max3_relu(P a, P b, P c) {
    return {__vimax3_s16x2_relu(a.v, b.v, c.v)};
  }
  __device__ __forceinline__ static P max3(P a, P b, P c) {
    return {__vimax3_s16x2(a.v, b.v, c.v)};
  }
  // max(a + b, c)
  __device__ __forceinline__ static P addmax(P a, P b, P c) {
    return {__viaddmax_s16x2(a.v, b.v, c.v)};
  }
  // Equality per lane as bit 15 (low) and bit 31 (high): a lane of x = a ^ b
  // is zero iff the values are equal; for a non-zero lane either x has its
  // top bit set or x + 0x7FFF does.  Three full-rate instructions (xor,
  // 16x2 add, one three-input logic op).
  __device__ __forceinline__ static uint32_t eqb(P a, P b) {
    const uint32_t x = a.v ^ b.v;
    return ~(__vadd2(x, 0x7FFF7FFFu) | x) & 0x80008000u;
  }
  __device__ __forceinline__ static P select(uint32_t m, P a, P b) {
    return {(a.v & m) | (b.v & ~m)};
  }
  // Substitution score of a pair of read characters (16-bit lanes holding
  // bytes) against row character rc2: m where equal, n elsewhere.  A lane of
  // (x ^ rc2) - 1 is 0xFFFF iff the characters are equal and below 0x00FF
  // otherwise; prmt replicates the sign of its high byte over the lane.
  __device__ __forceinline__ static P profile(uint32_t chars2, uint32_t rc2, P m2, P n2) {
    const uint32_t y = __vadd2(chars2 ^ rc2, 0xFFFFFFFFu);
    uint32_t mask;
#ifdef __CUDA_ARCH__
    asm("prmt.b32 %0, %1, 0, 0xBB99;" : "=r"(mask) : "r"(y));
#else  // host builds of this header (test harness): the same lane masks
    mask = ((y & 0x8000u) ? 0x0000FFFFu : 0u) | ((y & 0x80000000u) ? 0xFFFF0000u : 0u);
#endif
    return select(mask, m2, n2);
  }
  // 2 pairs per 8-byte access
  __device__ __forceinline__ static void load2(const void* base, uint64_t w, P& a, P& b) {
    uint2 x = reinterpret_cast<const uint2*>(base)[w >> 1];
    a.v = x.x;
    b.v = x.y;
  }
  __device__ __forceinline__ static void store2(void* base, uint64_t w, P a, P b) {
    reinterpret_cast<uint2*>(base)[w >> 1] = make_uint2(a.v, b.v);
  }
  // for rows only the traceback reads again (E, Q): evict-first, so they do
  // not push predecessor rows and graph data out of L2 (2.3 % faster on the
  // 10,000-window polishing batch)
  __device__ __forceinline__ static void store2cs(void* base, uint64_t w, P a, P b) {
    __stcs(reinterpret_cast<uint2*>(base) + (w >> 1), make_uint2(a.v, b.v));
  }
  __device__ __forceinline__ static int32_t elem(const void* base, uint64_t i) {
    return reinterpret_cast<const int16_t*>(base)[i];
  }
};

template <>
struct Lanes<int32_t> {
  struct P {
    int32_t l, h;
  };
  static constexpr int32_t kNeg = kNegBig;
  __device__ __forceinline__ static P make(int32_t lo, int32_t hi) { return {lo, hi}; }
  __device__ __forceinline__ static P splat(int32_t x) { return {x, x}; }
  __device__ __forceinline__ static int32_t lo(P a) { return a.l; }
  __device__ __forceinline__ static int32_t hi(P a) { return a.h; }
  __device__ __forceinline__ static P add(P a, P b) { return {a.l + b.l, a.h + b.h}; }
  __device__ __forceinline__ static P max(P a, P b, uint32_t) {
    return {a.l > b.l ? a.l : b.l, a.h > b.h ? a.h : b.h};
  }
  __device__ __forceinline__ static P max3_relu(P a, P b, P c) {
    return {__vimax3_s32_relu(a.l, b.l, c.l), __vimax3_s32_relu(a.h, b.h, c.h)};
  }
  __device__ __forceinline__ static P max3(P a, P b, P c) {
    return {__vimax3_s32(a.l, b.l, c.l), __vimax3_s32(a.h, b.h, c.h)};
  }
  __device__ __forceinline__ static P addmax(P a, P b, P c) {
    return {__viaddmax_s32(a.l, b.l, c.l), __viaddmax_s32(a.h, b.h, c.h)};
  }
  __device__ __forceinline__ static uint32_t eqb(P a, P b) {
    return (a.l == b.l ? 0x00008000u : 0u) | (a.h == b.h ? 0x80000000u : 0u);
  }
  __device__ __forceinline__ static P select(uint32_t m, P a, P b) {
    return {(m & 0xFFFFu) ? a.l : b.l, (m & 0xFFFF0000u) ? a.h : b.h};
  }
  __device__ __forceinline__ static P profile(uint32_t chars2, uint32_t rc2, P m2, P n2) {
    return {(chars2 & 0xFFFFu) == (rc2 & 0xFFFFu) ? m2.l : n2.l,
            (chars2 >> 16) == (rc2 >> 16) ? m2.h : n2.h};
  }
  __device__ __forceinline__ static void load2(const void* base, uint64_t w, P& a, P& b) {
    int4 x = reinterpret_cast<const int4*>(base)[w >> 1];
    a = {x.x, x.y};
    b = {x.z, x.w};
  }
  __device__ __forceinline__ static void store2(void* base, uint64_t w, P a, P b) {
    reinterpret_cast<int4*>(base)[w >> 1] = make_int4(a.l, a.h, b.l, b.h);
  }
  // int32 rows keep the default policy (not measured with the hint)
  __device__ __forceinline__ static void store2cs(void* base, uint64_t w, P a, P b) {
    store2(base, w, a, b);
  }
  __device__ __forceinline__ static int32_t elem(const void* base, uint64_t i) {
    return reinterpret_cast<const int32_t*>(base)[i];
  }
};

// Lane masks of a pair from two bits: 0xFFFF in the low lane when bit 15 of
// y is set, in the high lane when bit 31 is (one byte permute replicating
// the sign bits of bytes 1 and 3).
__device__ __forceinline__ uint32_t sign_lanes(uint32_t y) {
  uint32_t mask;
#ifdef __CUDA_ARCH__
  asm("prmt.b32 %0, %1, 0, 0xBB99;" : "=r"(mask) : "r"(y));
#else  // host builds of this header (test harness): the same lane masks
  mask = ((y & 0x8000u) ? 0x0000FFFFu : 0u) | ((y & 0x80000000u) ? 0xFFFF0000u : 0u);
#endif
  return mask;
}

// Element index of column j in a row of a CTA of nt threads (see DpView):
// column j is lane r / (CPT/2) of pair k = r % (CPT/2) of thread t = j / CPT
// (r = j % CPT), and pair k of thread t is pair word
// (k / 2) * 2 * nt + 2 * t + k % 2.
template <int CPT>
__host__ __device__ __forceinline__ uint64_t colmap(uint64_t j, uint64_t nt) {
  const uint64_t t = j / CPT, r = j % CPT, k = r % (CPT / 2);
  return 2 * ((k >> 1) * 2 * nt + 2 * t + (k & 1)) + r / (CPT / 2);
}

// Value of thread t-1 (thread 0 gets `fill`); the slots of sh.wv2 must not
// be written again before the CTA's next barrier.
template <int NW = 0>
__device__ __forceinline__ int32_t from_left(int32_t a, int32_t fill, BlockScratch& sh) {
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int32_t x = __shfl_up_sync(0xffffffffu, a, 1);
  if ((NW ? NW : blockDim.x >> 5) > 1) {
    if (lane == 31) sh.wv2[warp] = a;
    __syncthreads();
    if (lane == 0 && warp > 0) x = sh.wv2[warp - 1];
  }
  return threadIdx.x == 0 ? fill : x;
}

// Strip scan of X[j] = max(a[j], X[j-1] + pen) over this thread's pairs with
// the CTA carry.  On return x[k] holds X at the columns of pair k; returns
// X[s-1], the value carried into the strip (init for thread 0).
template <int CPT, typename Lx, int NW = 0>
__device__ __forceinline__ int32_t pair_scan(typename Lx::P* x, int32_t init, int32_t pen,
                                             int32_t* slots) {
  constexpr int HP = CPT / 2;
  static_assert(HP <= 16, "pair masks hold at most 16 pairs per strip");
  using P = typename Lx::P;
  const P pen2 = Lx::splat(pen);
#pragma unroll
  for (int k = 1; k < HP; ++k) x[k] = Lx::addmax(x[k - 1], pen2, x[k]);
  const int32_t lo_agg = Lx::lo(x[HP - 1]), hi_agg = Lx::hi(x[HP - 1]);
  const int32_t agg = imax(hi_agg, lo_agg + HP * pen);
  const int32_t c = scan_carry<CPT, NW>(agg, init, pen, slots);  // X[s-1]
  const int32_t c_hi = imax(lo_agg, c + HP * pen);          // X[s+HP-1]
  const P carry = Lx::make(c, c_hi);
#pragma unroll
  for (int k = 0; k < HP; ++k) x[k] = Lx::addmax(carry, Lx::splat((k + 1) * pen), x[k]);
  return c;
}

// The best path of a Q' carry into E' at column u of a CTA's range (u
// from 0): through a vector start u' <= u (u' + 1 a multiple of `lanes`,
// where E' also takes Q), at u' * c + (u - u') * e; linear in u', so the
// last vector start when c >= e, else the first.  -infinity before the
// first vector start.
__device__ __forceinline__ int32_t mq_path(int32_t u, int32_t c, int32_t e, int32_t lanes) {
  if (u < lanes - 1) return kNegBig;
  const int32_t up = c >= e ? ((u + 1) & ~(lanes - 1)) - 1 : lanes - 1;
  return up * c + (u - up) * e;
}

// What a cluster row carries into a CTA's range: the scan (H' for linear
// gaps, E' otherwise) and Q' (convex) at the column before the range, and H
// there (the diagonal source of the range's first column in the next row).
struct ClusterCarry {
  int32_t x, q, left;
};

// The one exchange of a cluster row, in two halves around the barrier so
// that work between them (the row's F/O stores) is not waited for.
// cluster_publish: the CTA's last thread publishes the CTA-local scans at
// the last two columns of its range (sa, sp; convex also Q': qa, qp) and h
// at the last column (ha), and every thread arrives.  The buffer alternates
// with the row parity: a CTA rewrites it two rows later, after a barrier
// that every CTA reaches only when done reading it.
template <int CL>
__device__ __forceinline__ void cluster_publish(int32_t sa, int32_t sp, int32_t ha, int32_t qa,
                                                int32_t qp, uint32_t row, BlockScratch& sh) {
  int32_t* rec = sh.clx[row & 1];
  if (threadIdx.x == blockDim.x - 1) {
    rec[0] = sa;
    rec[1] = sp;
    rec[2] = ha;
    rec[3] = qa;
    rec[4] = qp;
  }
  cl_arrive<CL>();
}

// cluster_fold: waits for the cluster, then every warp folds the CTAs
// before its own, lane k holding CTA k's values (X the carry into CTA k):
//   X'   = max(sa_k, X + W*pen)
//   E'   gains Q + g + mq_path(u)      (convex)
//   Q''  = max(qa_k, Q + W*c)
//   H    = max(ha_k, E'[W-2], Q'[W-2]) at CTA k's last column (relu for SW).
template <int SUB, int CL>
__device__ __forceinline__ ClusterCarry cluster_fold(uint32_t row, int32_t W, int32_t type,
                                                     int32_t pen, int32_t g, int32_t c, int32_t e,
                                                     int32_t lanes, BlockScratch& sh) {
  cl_wait<CL>();
  const int32_t* rec = sh.clx[row & 1];
  const uint32_t rank = cl_rank<CL>(), lane = threadIdx.x & 31;
  int32_t va = kNegBig, vp = kNegBig, vh = kNegBig, vqa = kNegBig, vqp = kNegBig;
  if (lane < rank) {
    va = cl_peek(rec + 0, lane);
    vp = cl_peek(rec + 1, lane);
    vh = cl_peek(rec + 2, lane);
    if (SUB == kConvex) {
      vqa = cl_peek(rec + 3, lane);
      vqp = cl_peek(rec + 4, lane);
    }
  }
  ClusterCarry r{kNegBig, kNegBig, 0};
  const int32_t mq_last = mq_path(W - 1, c, e, lanes), mq_prev = mq_path(W - 2, c, e, lanes);
  for (uint32_t k = 0; k < rank; ++k) {
    const int32_t a = __shfl_sync(0xffffffffu, va, k);
    const int32_t ap = __shfl_sync(0xffffffffu, vp, k);
    const int32_t ah = __shfl_sync(0xffffffffu, vh, k);
    int32_t xl = imax(a, r.x + W * pen), xp = imax(ap, r.x + (W - 1) * pen);
    int32_t ql = kNegBig, qpl = kNegBig;
    if (SUB == kConvex) {
      const int32_t aq = __shfl_sync(0xffffffffu, vqa, k);
      const int32_t aqp = __shfl_sync(0xffffffffu, vqp, k);
      ql = imax(aq, r.q + W * c);
      qpl = imax(aqp, r.q + (W - 1) * c);
      xl = imax(xl, r.q + g + mq_last);
      xp = imax(xp, r.q + g + mq_prev);
    }
    int32_t hl = SUB == kLinear ? xl : (SUB == kAffine ? imax(ah, xp) : imax(ah, imax(xp, qpl)));
    if (type == kSW) hl = imax(hl, 0);
    r.x = xl;
    r.q = ql;
    r.left = hl;
  }
  return r;
}


// Forward pass + row selection + max_j (identical in every thread on
// return).  T = int16_t for the 16-lane width, int32_t for the 8-lane one.
// NT: the CTA's threads when known at compile time (0: blockDim.x); with it
// every row offset of a load or store is a constant of the instruction and
// the scans of a one-warp CTA take no shared-memory path.
template <int SUB, int CPT, typename T, int NT = 0>
__device__ __noinline__ void dp_forward(const Scoring& S, DpView& D, const uint8_t* __restrict__ seq,
                           uint32_t L, uint32_t V, int32_t lanes, BlockScratch& sh,
                           int64_t* out_max_i, int64_t* out_max_j, int32_t* out_score) {
  using Lx = Lanes<T>;
  using P = typename Lx::P;
  using L16 = Lanes<int16_t>;
  constexpr int HP = CPT / 2;
  static_assert(HP <= 16, "pair masks hold at most 16 pairs per strip");
  const uint32_t t = threadIdx.x;
  const uint32_t s0 = t * CPT;
  const uint64_t ld = D.caps.ld;        // elements per row
  const uint64_t wrow = ld / 2;         // pair words per row
  // pairs k and k+1 (k even) of this thread: pair words w0 + (k/2) * st2
  // and the next; the warp's accesses to them are contiguous
  const uint64_t w0 = 2 * (uint64_t)t;
  constexpr int NW = NT / 32;
  const uint64_t st2 = 2 * (uint64_t)(NT ? NT : blockDim.x);
  const int32_t type = S.type;
  const int32_t m = S.m, n = S.n, g = S.g, e = S.e, q = S.q, c = S.c;
  const int32_t NEGW = lanes == 8 ? (INT32_MIN + 1024) : (INT16_MIN + 1024);
  void* __restrict__ H = D.H;
  void* __restrict__ F = D.F;
  void* __restrict__ O = D.O;
  void* __restrict__ E = D.E;
  void* __restrict__ Q = D.Q;
  const P NEG2 = Lx::splat(Lx::kNeg);
  const uint32_t NZ = S.min16x2;  // neutral operand of Lx::max
  const P m2 = Lx::splat(m), n2 = Lx::splat(n);
  const P g2 = Lx::splat(g), e2 = Lx::splat(e), q2 = Lx::splat(q), c2 = Lx::splat(c);
  const P ge2 = Lx::splat(g - e), qc2 = Lx::splat(q - c);
  const bool edge_thread = s0 + CPT > L;  // strip reaches past the read

  // read characters, 4 per register: byte b of sq8[k/4] is column s0+k of
  // the low half-strip (k = 4*(k/4) + b), sqh8 the same for the high half;
  // columns past the read hold 0xFF (whatever they match only feeds columns
  // past the read)
  uint32_t sq8[(HP + 3) / 4], sqh8[(HP + 3) / 4];
#pragma unroll
  for (int k4 = 0; k4 < (HP + 3) / 4; ++k4) {
    uint32_t lo = 0, hi = 0;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const uint32_t k = k4 * 4 + b;
      const uint32_t jl = s0 + k, jh = s0 + HP + k;
      lo |= (k < HP && jl < L ? (uint32_t)seq[jl] : 0xFFu) << (8 * b);
      hi |= (k < HP && jh < L ? (uint32_t)seq[jh] : 0xFFu) << (8 * b);
    }
    sq8[k4] = lo;
    sqh8[k4] = hi;
  }
  // the two characters of pair k as 16-bit lanes
  auto sq = [&](int k) -> L16::P {
    return L16::P{__byte_perm(sq8[k / 4], sqh8[k / 4], (uint32_t)(k % 4) | (0x4u + k % 4) << 8) &
                  0x00FF00FFu};
  };
  // convex: columns whose E' input also takes Q (vector starts of the
  // reference, (col + 1) % lanes == 0), as a bitmap (bit k low, 16+k high)
  uint32_t bmap = 0;
  if (SUB == kConvex) {
#pragma unroll
    for (int k = 0; k < HP; ++k) {
      if ((s0 + k + 1) % (uint32_t)lanes == 0) bmap |= 1u << k;
      if ((s0 + HP + k + 1) % (uint32_t)lanes == 0) bmap |= 1u << (16 + k);
    }
  }

  // row 0 (implementation.hpp:555-694) and its registers
  P ph[HP], pf[HP], po[HP];
#pragma unroll
  for (int k = 0; k < HP; ++k) {
    int32_t v[2];
#pragma unroll
    for (int hf = 0; hf < 2; ++hf) {
      const int32_t j = (int32_t)(s0 + hf * HP + k);
      if (type == kSW) {
        v[hf] = 0;
      } else if (SUB == kConvex) {
        v[hf] = imax(g + j * e, q + j * c);
      } else if (SUB == kAffine) {
        v[hf] = g + j * e;
      } else {
        v[hf] = g + j * g;
      }
    }
    ph[k] = Lx::make(v[0], v[1]);
    pf[k] = NEG2;
    po[k] = NEG2;
  }
#pragma unroll
  for (int k = 0; k < HP; k += 2) {
    const uint64_t wk = w0 + (k / 2) * st2;
    Lx::store2(H, wk, ph[k], ph[k + 1]);
    if (SUB >= kAffine) Lx::store2(F, wk, pf[k], pf[k + 1]);
    if (SUB == kConvex) Lx::store2(O, wk, po[k], po[k + 1]);
  }
  int32_t left_prev;  // row i-1 at column s0-1 (thread 0: its first column)
  {
    const int32_t j = (int32_t)s0 - 1;
    int32_t v;
    if (type == kSW) {
      v = 0;
    } else if (SUB == kConvex) {
      v = imax(g + j * e, q + j * c);
    } else if (SUB == kAffine) {
      v = g + j * e;
    } else {
      v = g + j * g;
    }
    left_prev = t == 0 ? 0 : v;
  }
  if (t == 0) {
    D.fc[0] = 0;
    D.fcF[0] = 0;
    D.fcO[0] = 0;
  }
  int32_t bval = type == kSW ? 0 : (type == kOV ? kNegBig : NEGW);
  int32_t brow = -1;
  int32_t first_sink = -1;
  // the thread holding column L-1 (NW selection)
  const uint32_t jl = L - 1;
  const bool owns_last = jl >= s0 && jl < s0 + CPT;
  const int32_t last_k = (int32_t)((jl - s0) % HP), last_hi = (int32_t)((jl - s0) / HP);
  // first column of the previous row (thread 0), kept in registers
  int32_t fc_prev = 0, fcF_prev = 0, fcO_prev = 0;
  // the next row's record is loaded one row ahead, off the critical path
  uint4 rec_next = D.rowrec[1];
  __syncthreads();

  for (uint32_t i = 1; i <= V; ++i) {
    const uint4 rec = rec_next;
    if (i < V) rec_next = D.rowrec[i + 1];
    const uint32_t rflags = (rec.y >> 16) & 0xFFu;
    const L16::P rc2 = L16::splat(rec.y >> 24);
    // Over the predecessors only maxima are taken: the diagonal source
    // max_p H_p[j-1] (hd), for linear gaps the vertical max_p H_p[j] (f),
    // for affine/convex max_p max(H_p + g - e, F_p) (f) and
    // max_p max(H_p + q - c, O_p) (o).  The substitution score and the gap
    // extension are the same for every predecessor and are added once per
    // row; max_p(x_p) + s = max_p(x_p + s) exactly (no value wraps: the width
    // rule keeps every finite value and the -infinity margin in range).
    P hd[HP], f[HP], o[HP];
    int32_t fl = kNegBig, fa = kNegBig, fo = kNegBig;
    // the predecessor order only matters to the traceback, which keeps the
    // reference's order
    auto accumulate = [&](const P* hp, const P* fp, const P* op, int32_t hleft, bool first) {
#pragma unroll
      for (int k = 0; k < HP; ++k) {
        const P left = k == 0 ? Lx::make(hleft, Lx::lo(hp[HP - 1])) : hp[k - 1];
        hd[k] = first ? left : Lx::max(hd[k], left, NZ);
        if (SUB == kLinear) {
          f[k] = first ? hp[k] : Lx::max(f[k], hp[k], NZ);
        } else {
          f[k] = first ? Lx::addmax(hp[k], ge2, fp[k]) : Lx::max3(f[k], Lx::add(hp[k], ge2), fp[k]);
          if (SUB == kConvex)
            o[k] = first ? Lx::addmax(hp[k], qc2, op[k]) : Lx::max3(o[k], Lx::add(hp[k], qc2), op[k]);
        }
      }
    };
    bool first = true;
    if (rflags & kRowPrevPred) {
      // the previous rank is a predecessor: its row is in registers
      if (t == 0) {
        fl = imax(fl, fc_prev);
        if (SUB >= kAffine) fa = imax(fa, fcF_prev);
        if (SUB == kConvex) fo = imax(fo, fcO_prev);
      }
      accumulate(ph, pf, po, t == 0 ? fc_prev : left_prev, true);
      first = false;
    }
    // the other predecessors: two from the record, any further ones from the
    // predecessor list (rows with more than two are rare)
    uint32_t p = rec.z;
    uint32_t visited = 0, skipped = 0;
    uint32_t pi = rec.x;
    const uint32_t pend = (rflags & kRowMore) ? D.pred_ptr[i + 1] : rec.x;
    while (p != kNone) {
      P hp[HP], fp[HP], op[HP];
      const uint64_t rwp = (uint64_t)p * wrow + w0;
#pragma unroll
      for (int k = 0; k < HP; k += 2) {
        const uint64_t wk = rwp + (k / 2) * st2;
        Lx::load2(H, wk, hp[k], hp[k + 1]);
        if (SUB >= kAffine) Lx::load2(F, wk, fp[k], fp[k + 1]);
        if (SUB == kConvex) Lx::load2(O, wk, op[k], op[k + 1]);
      }
      // column s0-1: the high lane of the left thread's last pair (HP-1,
      // odd), pair word (HP/2 - 1) * st2 + w0 - 1
      int32_t hleft;
      if (t == 0) {
        hleft = D.fc[p];
        fl = imax(fl, D.fc[p]);
        if (SUB >= kAffine) fa = imax(fa, D.fcF[p]);
        if (SUB == kConvex) fo = imax(fo, D.fcO[p]);
      } else {
        hleft = Lx::elem(H, (uint64_t)p * ld + 2 * ((HP / 2 - 1) * st2 + w0 - 1) + 1);
      }
      accumulate(hp, fp, op, hleft, first);
      first = false;
      if (++visited == 1) {
        p = rec.w;
      } else {
        p = kNone;
        while (pi < pend) {
          const uint32_t q = D.preds[pi++];
          if (q == i - 1) continue;
          if (skipped < 2) {
            ++skipped;
            continue;
          }
          p = q;
          break;
        }
      }
    }
    // NW first column (thread 0)
    int32_t fci = 0;
    if (t == 0) {
      const bool source = (rflags & kRowSource) != 0;
      if (type == kNW) {
        if (SUB == kLinear) {
          fci = (source ? 0 : fl) + g;
        } else {
          const int32_t vF = (source ? g - e : fa) + e;
          D.fcF[i] = vF;
          fcF_prev = vF;
          if (SUB == kConvex) {
            const int32_t vO = (source ? q - c : fo) + c;
            D.fcO[i] = vO;
            fcO_prev = vO;
            fci = imax(vF, vO);
          } else {
            fci = vF;
          }
        }
      }
      D.fc[i] = fci;
      fc_prev = fci;
    }
    const uint64_t rw = (uint64_t)i * wrow + w0;
    P h[HP];
#pragma unroll
    for (int k = 0; k < HP; ++k) {
      const P d = Lx::add(hd[k], Lx::profile(sq(k).v, rc2.v, m2, n2));
      if (SUB == kLinear) {
        h[k] = Lx::addmax(f[k], g2, d);
      } else {
        f[k] = Lx::add(f[k], e2);
        if (SUB == kConvex) {
          o[k] = Lx::add(o[k], c2);
          h[k] = Lx::max3(d, f[k], o[k]);
        } else {
          h[k] = Lx::max(d, f[k], NZ);
        }
      }
    }
    if (SUB >= kAffine) {
#pragma unroll
      for (int k = 0; k < HP; k += 2) {
        Lx::store2(F, rw + (k / 2) * st2, f[k], f[k + 1]);
        if (SUB == kConvex) Lx::store2(O, rw + (k / 2) * st2, o[k], o[k + 1]);
      }
    }
    // Columns past the read are computed like the others and never masked:
    // they only feed columns to their right (the in-row scans run left to
    // right, the diagonal reads column j-1), the row selection below masks
    // them, and the traceback never reaches them.
    P hs[HP], ee[HP], qq[HP];
    if (SUB == kLinear) {
#pragma unroll
      for (int k = 0; k < HP; ++k) hs[k] = h[k];
      pair_scan<CPT, Lx, NW>(hs, fci, g, sh.wv);
      if (type == kSW) {
        const P z = Lx::splat(0);
#pragma unroll
        for (int k = 0; k < HP; ++k) hs[k] = Lx::max(hs[k], z, NZ);
      }
    } else {
      if (SUB == kConvex) {
        P x[HP];
#pragma unroll
        for (int k = 0; k < HP; ++k) x[k] = Lx::add(h[k], q2);
        // x = Q' (Q of the next column); Q[s0] = Q'[s0-1] is the carry
        const int32_t qin = pair_scan<CPT, Lx, NW>(x, fci + q, c, sh.wq);
        qq[0] = Lx::make(qin, Lx::lo(x[HP - 1]));
#pragma unroll
        for (int k = 1; k < HP; ++k) qq[k] = x[k - 1];
      }
      {
        P x[HP];
#pragma unroll
        for (int k = 0; k < HP; ++k) {
          if (SUB == kConvex) {
            // max(H1, Q at vector starts) + g: bits k and 16 + k of bmap
            // moved to bits 15 and 31 give the pair's lane masks
            const uint32_t bm = sign_lanes(bmap << (15 - k));
            x[k] = Lx::add(Lx::max(h[k], Lx::select(bm, qq[k], NEG2), NZ), g2);
          } else {
            x[k] = Lx::add(h[k], g2);
          }
        }
        const int32_t ein = pair_scan<CPT, Lx, NW>(x, fci + g, e, sh.wv);  // x = E'
        ee[0] = Lx::make(ein, Lx::lo(x[HP - 1]));
#pragma unroll
        for (int k = 1; k < HP; ++k) ee[k] = x[k - 1];
      }
#pragma unroll
      for (int k = 0; k < HP; ++k) {
        if (SUB == kConvex)
          hs[k] = type == kSW ? Lx::max3_relu(h[k], ee[k], qq[k]) : Lx::max3(h[k], ee[k], qq[k]);
        else
          hs[k] = type == kSW ? Lx::max3_relu(h[k], ee[k], ee[k]) : Lx::max(h[k], ee[k], NZ);
      }
    }
    // column s0-1 of this row (thread 0: the first column fc)
    const int32_t lH = from_left<NW>(Lx::hi(hs[HP - 1]), fci, sh);
    // the gap rows E and Q as the recurrences computed them: the traceback
    // re-derives its horizontal tests from them
    if (SUB >= kAffine) {
#pragma unroll
      for (int k = 0; k < HP; k += 2) {
        Lx::store2cs(E, rw + (k / 2) * st2, ee[k], ee[k + 1]);
        if (SUB == kConvex) Lx::store2cs(Q, rw + (k / 2) * st2, qq[k], qq[k + 1]);
      }
    }
#pragma unroll
    for (int k = 0; k < HP; k += 2) Lx::store2(H, rw + (k / 2) * st2, hs[k], hs[k + 1]);

    // row selection (strict <: the earliest row wins a tie)
    if (type == kNW) {
      if ((rflags & kRowSink) && owns_last) {
        int32_t v = kNegBig;
#pragma unroll
        for (int k = 0; k < HP; ++k)
          if (k == last_k) v = last_hi ? Lx::hi(hs[k]) : Lx::lo(hs[k]);
        if (v > bval) {
          bval = v;
          brow = (int32_t)i;
        }
      }
    } else if (type == kSW || (rflags & kRowSink)) {
      P mx = hs[0];
      if (edge_thread) {
#pragma unroll
        for (int k = 0; k < HP; ++k) {
          const uint32_t vm = (s0 + k < L ? 0x0000FFFFu : 0u) | (s0 + HP + k < L ? 0xFFFF0000u : 0u);
          const P x = Lx::select(vm, hs[k], NEG2);
          mx = k == 0 ? x : Lx::max(mx, x, NZ);
        }
      } else {
#pragma unroll
        for (int k = 1; k < HP; ++k) mx = Lx::max(mx, hs[k], NZ);
      }
      const int32_t tm = s0 < L ? imax(Lx::lo(mx), Lx::hi(mx)) : kNegBig;
      if (tm > bval) {
        bval = tm;
        brow = (int32_t)i;
      }
      if (type == kOV && first_sink < 0) first_sink = (int32_t)i;
    }
    // this row becomes the registers of row i-1
#pragma unroll
    for (int k = 0; k < HP; ++k) {
      ph[k] = hs[k];
      if (SUB >= kAffine) pf[k] = f[k];
      if (SUB == kConvex) po[k] = o[k];
    }
    left_prev = t == 0 ? 0 : lH;
    __syncthreads();
  }

  // global selection: best value, then the earliest row reaching it
  const int32_t B = block_max<NW>(bval, sh);
  const int32_t R = block_min<NW>(bval == B && brow >= 0 ? brow : 0x7fffffff, sh);
  int64_t max_i = -1;
  int32_t score = 0;
  if (type == kSW) {
    if (B > 0 && R != 0x7fffffff) {
      max_i = R;
      score = B;
    }
  } else if (type == kOV) {
    // _mmxxx_max_value starts from 0: a sink row never scores below 0, and
    // when no sink row is positive the first sink row wins with score 0
    if (B > 0) {
      max_i = R;
      score = B;
    } else {
      max_i = first_sink;
      score = 0;
    }
  } else {
    if (R != 0x7fffffff && B > NEGW) {
      max_i = R;
      score = B;
    }
  }
  int64_t max_j = -1;
  if (max_i >= 0) {
    if (type == kNW) {
      max_j = (int64_t)L - 1;
    } else {
      const uint64_t base = (uint64_t)max_i * ld;
      int32_t jj = 0x7fffffff;
      for (int r = 0; r < CPT && jj == 0x7fffffff; ++r) {
        const uint32_t j = s0 + r;
        if (j < L && Lx::elem(H, base + colmap<CPT>(j, NT ? NT : blockDim.x)) == score) jj = (int32_t)j;
      }
      jj = block_min<NW>(jj, sh);
      max_j = jj == 0x7fffffff ? -1 : jj;
    }
  }
  *out_max_i = max_i;
  *out_max_j = max_j;
  *out_score = score;
}

// The forward pass of dp_forward over a thread-block cluster of CL CTAs
// (long 32-bit rows): CTA r of the cluster owns virtual threads
// r * nt ... r * nt + nt - 1 of the row, and the in-row scans cross the CTAs
// through one exchange per row (cluster_publish / cluster_fold).  Its own
// function, apart from dp_forward: the one-CTA forward is the polishing
// batch's hot loop, and a shared template measurably changed its code.
template <int SUB, int CPT, typename T, int CL>
__device__ __noinline__ void dp_forward_cl(const Scoring& S, DpView& D,
                                           const uint8_t* __restrict__ seq, uint32_t L,
                                           uint32_t V, int32_t lanes, BlockScratch& sh,
                                           int64_t* out_max_i, int64_t* out_max_j,
                                           int32_t* out_score) {
  static_assert(CL > 1, "one CTA runs dp_forward");
  constexpr int NT = 0;
  using Lx = Lanes<T>;
  using P = typename Lx::P;
  using L16 = Lanes<int16_t>;
  constexpr int HP = CPT / 2;
  static_assert(HP <= 16, "pair masks hold at most 16 pairs per strip");
  // this thread's index in the cluster's row
  const uint32_t ntc = NT ? NT : blockDim.x;  // threads of the CTA
  const uint32_t ntv = ntc * CL;               // threads of the row
  const uint32_t t = cl_rank<CL>() * ntc + threadIdx.x;
  const uint32_t s0 = t * CPT;
  const uint64_t ld = D.caps.ld;        // elements per row
  const uint64_t wrow = ld / 2;         // pair words per row
  // pairs k and k+1 (k even) of this thread: pair words w0 + (k/2) * st2
  // and the next; the warp's accesses to them are contiguous
  const uint64_t w0 = 2 * (uint64_t)t;
  constexpr int NW = NT / 32;
  const uint64_t st2 = 2 * (uint64_t)ntv;
  const int32_t type = S.type;
  const int32_t m = S.m, n = S.n, g = S.g, e = S.e, q = S.q, c = S.c;
  const int32_t NEGW = lanes == 8 ? (INT32_MIN + 1024) : (INT16_MIN + 1024);
  void* __restrict__ H = D.H;
  void* __restrict__ F = D.F;
  void* __restrict__ O = D.O;
  void* __restrict__ E = D.E;
  void* __restrict__ Q = D.Q;
  const P NEG2 = Lx::splat(Lx::kNeg);
  const uint32_t NZ = S.min16x2;  // neutral operand of Lx::max
  const P m2 = Lx::splat(m), n2 = Lx::splat(n);
  const P g2 = Lx::splat(g), e2 = Lx::splat(e), q2 = Lx::splat(q), c2 = Lx::splat(c);
  const P ge2 = Lx::splat(g - e), qc2 = Lx::splat(q - c);
  const bool edge_thread = s0 + CPT > L;  // strip reaches past the read

  // read characters, 4 per register: byte b of sq8[k/4] is column s0+k of
  // the low half-strip (k = 4*(k/4) + b), sqh8 the same for the high half;
  // columns past the read hold 0xFF (whatever they match only feeds columns
  // past the read)
  uint32_t sq8[(HP + 3) / 4], sqh8[(HP + 3) / 4];
#pragma unroll
  for (int k4 = 0; k4 < (HP + 3) / 4; ++k4) {
    uint32_t lo = 0, hi = 0;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const uint32_t k = k4 * 4 + b;
      const uint32_t jl = s0 + k, jh = s0 + HP + k;
      lo |= (k < HP && jl < L ? (uint32_t)seq[jl] : 0xFFu) << (8 * b);
      hi |= (k < HP && jh < L ? (uint32_t)seq[jh] : 0xFFu) << (8 * b);
    }
    sq8[k4] = lo;
    sqh8[k4] = hi;
  }
  // the two characters of pair k as 16-bit lanes
  auto sq = [&](int k) -> L16::P {
    return L16::P{__byte_perm(sq8[k / 4], sqh8[k / 4], (uint32_t)(k % 4) | (0x4u + k % 4) << 8) &
                  0x00FF00FFu};
  };
  // convex: columns whose E' input also takes Q (vector starts of the
  // reference, (col + 1) % lanes == 0), as a bitmap (bit k low, 16+k high)
  uint32_t bmap = 0;
  if (SUB == kConvex) {
#pragma unroll
    for (int k = 0; k < HP; ++k) {
      if ((s0 + k + 1) % (uint32_t)lanes == 0) bmap |= 1u << k;
      if ((s0 + HP + k + 1) % (uint32_t)lanes == 0) bmap |= 1u << (16 + k);
    }
  }

  // row 0 (implementation.hpp:555-694) and its registers
  P ph[HP], pf[HP], po[HP];
#pragma unroll
  for (int k = 0; k < HP; ++k) {
    int32_t v[2];
#pragma unroll
    for (int hf = 0; hf < 2; ++hf) {
      const int32_t j = (int32_t)(s0 + hf * HP + k);
      if (type == kSW) {
        v[hf] = 0;
      } else if (SUB == kConvex) {
        v[hf] = imax(g + j * e, q + j * c);
      } else if (SUB == kAffine) {
        v[hf] = g + j * e;
      } else {
        v[hf] = g + j * g;
      }
    }
    ph[k] = Lx::make(v[0], v[1]);
    pf[k] = NEG2;
    po[k] = NEG2;
  }
#pragma unroll
  for (int k = 0; k < HP; k += 2) {
    const uint64_t wk = w0 + (k / 2) * st2;
    Lx::store2(H, wk, ph[k], ph[k + 1]);
    if (SUB >= kAffine) Lx::store2(F, wk, pf[k], pf[k + 1]);
    if (SUB == kConvex) Lx::store2(O, wk, po[k], po[k + 1]);
  }
  int32_t left_prev;  // row i-1 at column s0-1 (thread 0: its first column)
  {
    const int32_t j = (int32_t)s0 - 1;
    int32_t v;
    if (type == kSW) {
      v = 0;
    } else if (SUB == kConvex) {
      v = imax(g + j * e, q + j * c);
    } else if (SUB == kAffine) {
      v = g + j * e;
    } else {
      v = g + j * g;
    }
    left_prev = t == 0 ? 0 : v;
  }
  if (t == 0) {
    D.fc[0] = 0;
    D.fcF[0] = 0;
    D.fcO[0] = 0;
  }
  int32_t bval = type == kSW ? 0 : (type == kOV ? kNegBig : NEGW);
  int32_t brow = -1;
  int32_t first_sink = -1;
  // the thread holding column L-1 (NW selection)
  const uint32_t jl = L - 1;
  const bool owns_last = jl >= s0 && jl < s0 + CPT;
  const int32_t last_k = (int32_t)((jl - s0) % HP), last_hi = (int32_t)((jl - s0) / HP);
  // first column of the previous row (thread 0), kept in registers
  int32_t fc_prev = 0, fcF_prev = 0, fcO_prev = 0;
  // the next row's record is loaded one row ahead, off the critical path
  uint4 rec_next = D.rowrec[1];
  __syncthreads();

  for (uint32_t i = 1; i <= V; ++i) {
    const uint4 rec = rec_next;
    if (i < V) rec_next = D.rowrec[i + 1];
    const uint32_t rflags = (rec.y >> 16) & 0xFFu;
    const L16::P rc2 = L16::splat(rec.y >> 24);
    // Over the predecessors only maxima are taken: the diagonal source
    // max_p H_p[j-1] (hd), for linear gaps the vertical max_p H_p[j] (f),
    // for affine/convex max_p max(H_p + g - e, F_p) (f) and
    // max_p max(H_p + q - c, O_p) (o).  The substitution score and the gap
    // extension are the same for every predecessor and are added once per
    // row; max_p(x_p) + s = max_p(x_p + s) exactly (no value wraps: the width
    // rule keeps every finite value and the -infinity margin in range).
    P hd[HP], f[HP], o[HP];
    int32_t fl = kNegBig, fa = kNegBig, fo = kNegBig;
    // the predecessor order only matters to the traceback, which keeps the
    // reference's order
    auto accumulate = [&](const P* hp, const P* fp, const P* op, int32_t hleft, bool first) {
#pragma unroll
      for (int k = 0; k < HP; ++k) {
        const P left = k == 0 ? Lx::make(hleft, Lx::lo(hp[HP - 1])) : hp[k - 1];
        hd[k] = first ? left : Lx::max(hd[k], left, NZ);
        if (SUB == kLinear) {
          f[k] = first ? hp[k] : Lx::max(f[k], hp[k], NZ);
        } else {
          f[k] = first ? Lx::addmax(hp[k], ge2, fp[k]) : Lx::max3(f[k], Lx::add(hp[k], ge2), fp[k]);
          if (SUB == kConvex)
            o[k] = first ? Lx::addmax(hp[k], qc2, op[k]) : Lx::max3(o[k], Lx::add(hp[k], qc2), op[k]);
        }
      }
    };
    bool first = true;
    if (rflags & kRowPrevPred) {
      // the previous rank is a predecessor: its row is in registers
      if (t == 0) {
        fl = imax(fl, fc_prev);
        if (SUB >= kAffine) fa = imax(fa, fcF_prev);
        if (SUB == kConvex) fo = imax(fo, fcO_prev);
      }
      accumulate(ph, pf, po, t == 0 ? fc_prev : left_prev, true);
      first = false;
    }
    // the other predecessors: two from the record, any further ones from the
    // predecessor list (rows with more than two are rare)
    uint32_t p = rec.z;
    uint32_t visited = 0, skipped = 0;
    uint32_t pi = rec.x;
    const uint32_t pend = (rflags & kRowMore) ? D.pred_ptr[i + 1] : rec.x;
    while (p != kNone) {
      P hp[HP], fp[HP], op[HP];
      const uint64_t rwp = (uint64_t)p * wrow + w0;
#pragma unroll
      for (int k = 0; k < HP; k += 2) {
        const uint64_t wk = rwp + (k / 2) * st2;
        Lx::load2(H, wk, hp[k], hp[k + 1]);
        if (SUB >= kAffine) Lx::load2(F, wk, fp[k], fp[k + 1]);
        if (SUB == kConvex) Lx::load2(O, wk, op[k], op[k + 1]);
      }
      // column s0-1: the high lane of the left thread's last pair (HP-1,
      // odd), pair word (HP/2 - 1) * st2 + w0 - 1
      int32_t hleft;
      if (t == 0) {
        hleft = D.fc[p];
        fl = imax(fl, D.fc[p]);
        if (SUB >= kAffine) fa = imax(fa, D.fcF[p]);
        if (SUB == kConvex) fo = imax(fo, D.fcO[p]);
      } else {
        hleft = Lx::elem(H, (uint64_t)p * ld + 2 * ((HP / 2 - 1) * st2 + w0 - 1) + 1);
      }
      accumulate(hp, fp, op, hleft, first);
      first = false;
      if (++visited == 1) {
        p = rec.w;
      } else {
        p = kNone;
        while (pi < pend) {
          const uint32_t q = D.preds[pi++];
          if (q == i - 1) continue;
          if (skipped < 2) {
            ++skipped;
            continue;
          }
          p = q;
          break;
        }
      }
    }
    // NW first column (thread 0)
    int32_t fci = 0;
    if (t == 0) {
      const bool source = (rflags & kRowSource) != 0;
      if (type == kNW) {
        if (SUB == kLinear) {
          fci = (source ? 0 : fl) + g;
        } else {
          const int32_t vF = (source ? g - e : fa) + e;
          D.fcF[i] = vF;
          fcF_prev = vF;
          if (SUB == kConvex) {
            const int32_t vO = (source ? q - c : fo) + c;
            D.fcO[i] = vO;
            fcO_prev = vO;
            fci = imax(vF, vO);
          } else {
            fci = vF;
          }
        }
      }
      D.fc[i] = fci;
      fc_prev = fci;
    }
    const uint64_t rw = (uint64_t)i * wrow + w0;
    P h[HP];
#pragma unroll
    for (int k = 0; k < HP; ++k) {
      const P d = Lx::add(hd[k], Lx::profile(sq(k).v, rc2.v, m2, n2));
      if (SUB == kLinear) {
        h[k] = Lx::addmax(f[k], g2, d);
      } else {
        f[k] = Lx::add(f[k], e2);
        if (SUB == kConvex) {
          o[k] = Lx::add(o[k], c2);
          h[k] = Lx::max3(d, f[k], o[k]);
        } else {
          h[k] = Lx::max(d, f[k], NZ);
        }
      }
    }
    // the row's F and O (a cluster stores them while its barrier completes)
    auto store_fo = [&]() {
      if (SUB >= kAffine) {
#pragma unroll
        for (int k = 0; k < HP; k += 2) {
          Lx::store2(F, rw + (k / 2) * st2, f[k], f[k + 1]);
          if (SUB == kConvex) Lx::store2(O, rw + (k / 2) * st2, o[k], o[k + 1]);
        }
      }
    };
    // Columns past the read are computed like the others and never masked:
    // they only feed columns to their right (the in-row scans run left to
    // right, the diagonal reads column j-1), the row selection below masks
    // them, and the traceback never reaches them.
    P hs[HP], ee[HP], qq[HP];
    // column s0-1 of this row for the CTA's thread 0: the first column fc
    // in the cluster's first CTA, else the last column of the CTA before
    int32_t lfill = fci;
    {
      // A cluster row: CTA r owns columns r*W ... r*W + W - 1.  Every in-row
      // scan runs CTA-local, from the row's initial values in CTA 0 and from
      // -infinity in the others; one exchange then gives each CTA the values
      // carried into its range (cluster_fold).  The scans are max-plus
      // linear, so a carry X of a scan with penalty pen adds
      // X + (u + 1) * pen at column u of the range, and for convex gaps the
      // Q carry also reaches E' through the vector starts (mq_path).
      const uint32_t rank = cl_rank<CL>();
      const int32_t u0 = (int32_t)(threadIdx.x * CPT);  // first column in the range
      // linear: H'; affine, convex: E' (and Q' in xq)
      P xs[HP], xq[HP];
      int32_t qin = kNegBig, sc_in;
      if (SUB == kConvex) {
#pragma unroll
        for (int k = 0; k < HP; ++k) xq[k] = Lx::add(h[k], q2);
        qin = pair_scan<CPT, Lx, NW>(xq, rank == 0 ? fci + q : kNegBig, c, sh.wq);
        qq[0] = Lx::make(qin, Lx::lo(xq[HP - 1]));
#pragma unroll
        for (int k = 1; k < HP; ++k) qq[k] = xq[k - 1];
      }
#pragma unroll
      for (int k = 0; k < HP; ++k) {
        if (SUB == kLinear) {
          xs[k] = h[k];
        } else if (SUB == kConvex) {
          const uint32_t bm = sign_lanes(bmap << (15 - k));
          xs[k] = Lx::add(Lx::max(h[k], Lx::select(bm, qq[k], NEG2), NZ), g2);
        } else {
          xs[k] = Lx::add(h[k], g2);
        }
      }
      const int32_t pen = SUB == kLinear ? g : e;
      sc_in = pair_scan<CPT, Lx, NW>(xs, rank == 0 ? (SUB == kLinear ? fci : fci + g) : kNegBig,
                                     pen, sh.wv);
      cluster_publish<CL>(Lx::hi(xs[HP - 1]), Lx::hi(xs[HP - 2]), Lx::hi(h[HP - 1]),
                          SUB == kConvex ? Lx::hi(xq[HP - 1]) : kNegBig,
                          SUB == kConvex ? Lx::hi(xq[HP - 2]) : kNegBig, i, sh);
      store_fo();
      const ClusterCarry cc =
          cluster_fold<SUB, CL>(i, (int32_t)(ntc * CPT), type, pen, g, c, e, lanes, sh);
      if (rank > 0) {
        const P cs = Lx::make(cc.x + (u0 + 1) * pen, cc.x + (u0 + HP + 1) * pen);
#pragma unroll
        for (int k = 0; k < HP; ++k) xs[k] = Lx::addmax(cs, Lx::splat(k * pen), xs[k]);
        sc_in = imax(sc_in, cc.x + u0 * pen);
        if (SUB == kConvex) {
          const P cq = Lx::make(cc.q + (u0 + 1) * c, cc.q + (u0 + HP + 1) * c);
#pragma unroll
          for (int k = 0; k < HP; ++k) xq[k] = Lx::addmax(cq, Lx::splat(k * c), xq[k]);
          qin = imax(qin, cc.q + u0 * c);
          qq[0] = Lx::make(qin, Lx::lo(xq[HP - 1]));
#pragma unroll
          for (int k = 1; k < HP; ++k) qq[k] = xq[k - 1];
          const int32_t qg = cc.q + g;
#pragma unroll
          for (int k = 0; k < HP; ++k)
            xs[k] = Lx::max(xs[k], Lx::make(qg + mq_path(u0 + k, c, e, lanes),
                                            qg + mq_path(u0 + HP + k, c, e, lanes)), NZ);
          sc_in = imax(sc_in, qg + mq_path(u0 - 1, c, e, lanes));
        }
        lfill = cc.left;
      }
      if (SUB == kLinear) {
#pragma unroll
        for (int k = 0; k < HP; ++k) hs[k] = xs[k];
        if (type == kSW) {
          const P z = Lx::splat(0);
#pragma unroll
          for (int k = 0; k < HP; ++k) hs[k] = Lx::max(hs[k], z, NZ);
        }
      } else {
        ee[0] = Lx::make(sc_in, Lx::lo(xs[HP - 1]));
#pragma unroll
        for (int k = 1; k < HP; ++k) ee[k] = xs[k - 1];
#pragma unroll
        for (int k = 0; k < HP; ++k) {
          if (SUB == kConvex)
            hs[k] = type == kSW ? Lx::max3_relu(h[k], ee[k], qq[k]) : Lx::max3(h[k], ee[k], qq[k]);
          else
            hs[k] = type == kSW ? Lx::max3_relu(h[k], ee[k], ee[k]) : Lx::max(h[k], ee[k], NZ);
        }
      }
    }
    const int32_t lH = from_left<NW>(Lx::hi(hs[HP - 1]), lfill, sh);
    // the gap rows E and Q as the recurrences computed them: the traceback
    // re-derives its horizontal tests from them
    if (SUB >= kAffine) {
#pragma unroll
      for (int k = 0; k < HP; k += 2) {
        Lx::store2cs(E, rw + (k / 2) * st2, ee[k], ee[k + 1]);
        if (SUB == kConvex) Lx::store2cs(Q, rw + (k / 2) * st2, qq[k], qq[k + 1]);
      }
    }
#pragma unroll
    for (int k = 0; k < HP; k += 2) Lx::store2(H, rw + (k / 2) * st2, hs[k], hs[k + 1]);

    // row selection (strict <: the earliest row wins a tie)
    if (type == kNW) {
      if ((rflags & kRowSink) && owns_last) {
        int32_t v = kNegBig;
#pragma unroll
        for (int k = 0; k < HP; ++k)
          if (k == last_k) v = last_hi ? Lx::hi(hs[k]) : Lx::lo(hs[k]);
        if (v > bval) {
          bval = v;
          brow = (int32_t)i;
        }
      }
    } else if (type == kSW || (rflags & kRowSink)) {
      P mx = hs[0];
      if (edge_thread) {
#pragma unroll
        for (int k = 0; k < HP; ++k) {
          const uint32_t vm = (s0 + k < L ? 0x0000FFFFu : 0u) | (s0 + HP + k < L ? 0xFFFF0000u : 0u);
          const P x = Lx::select(vm, hs[k], NEG2);
          mx = k == 0 ? x : Lx::max(mx, x, NZ);
        }
      } else {
#pragma unroll
        for (int k = 1; k < HP; ++k) mx = Lx::max(mx, hs[k], NZ);
      }
      const int32_t tm = s0 < L ? imax(Lx::lo(mx), Lx::hi(mx)) : kNegBig;
      if (tm > bval) {
        bval = tm;
        brow = (int32_t)i;
      }
      if (type == kOV && first_sink < 0) first_sink = (int32_t)i;
    }
    // this row becomes the registers of row i-1
#pragma unroll
    for (int k = 0; k < HP; ++k) {
      ph[k] = hs[k];
      if (SUB >= kAffine) pf[k] = f[k];
      if (SUB == kConvex) po[k] = o[k];
    }
    left_prev = t == 0 ? 0 : lH;
    __syncthreads();
  }

  // global selection: best value, then the earliest row reaching it
  const int32_t B = cluster_max<NW, CL>(bval, sh, kClMax);
  const int32_t R = cluster_min<NW, CL>(bval == B && brow >= 0 ? brow : 0x7fffffff, sh, kClMin);
  int64_t max_i = -1;
  int32_t score = 0;
  if (type == kSW) {
    if (B > 0 && R != 0x7fffffff) {
      max_i = R;
      score = B;
    }
  } else if (type == kOV) {
    // _mmxxx_max_value starts from 0: a sink row never scores below 0, and
    // when no sink row is positive the first sink row wins with score 0
    if (B > 0) {
      max_i = R;
      score = B;
    } else {
      max_i = first_sink;
      score = 0;
    }
  } else {
    if (R != 0x7fffffff && B > NEGW) {
      max_i = R;
      score = B;
    }
  }
  int64_t max_j = -1;
  if (max_i >= 0) {
    if (type == kNW) {
      max_j = (int64_t)L - 1;
    } else {
      const uint64_t base = (uint64_t)max_i * ld;
      int32_t jj = 0x7fffffff;
      for (int r = 0; r < CPT && jj == 0x7fffffff; ++r) {
        const uint32_t j = s0 + r;
        if (j < L && Lx::elem(H, base + colmap<CPT>(j, ntv)) == score) jj = (int32_t)j;
      }
      jj = cluster_min<NW, CL>(jj, sh, kClMinJ);
      max_j = jj == 0x7fffffff ? -1 : jj;
    }
  }
  *out_max_i = max_i;
  *out_max_j = max_j;
  *out_score = score;
}

// Forward pass for rows longer than one strip per thread can hold: thread t
// owns SEGS strips of CPT columns, strip g being virtual thread g*nt + t of
// a CTA of SEGS*nt virtual threads (the row layout and colmap use that
// width).  Per row the strips are processed left to right; every scan of a
// strip starts from the carry of the strip before it (passed through shared
// memory from its last thread), and the previous row is read back from
// memory like any other predecessor instead of being kept in registers.
// Same results as dp_forward, cell by cell.
template <int SUB, int CPT, typename T, int SEGS>
__device__ __noinline__ void dp_forward_seg(const Scoring& S, DpView& D,
                                            const uint8_t* __restrict__ seq, uint32_t L,
                                            uint32_t V, int32_t lanes, BlockScratch& sh,
                                            int64_t* out_max_i, int64_t* out_max_j,
                                            int32_t* out_score) {
  using Lx = Lanes<T>;
  using P = typename Lx::P;
  using L16 = Lanes<int16_t>;
  constexpr int HP = CPT / 2;
  static_assert(HP <= 16, "pair masks hold at most 16 pairs per strip");
  const uint32_t t = threadIdx.x, nt = blockDim.x, ntv = nt * SEGS;
  const uint64_t ld = D.caps.ld;
  const uint64_t wrow = ld / 2;
  const uint64_t st2 = 2 * (uint64_t)ntv;
  const int32_t type = S.type;
  const int32_t m = S.m, n = S.n, g = S.g, e = S.e, q = S.q, c = S.c;
  const int32_t NEGW = lanes == 8 ? (INT32_MIN + 1024) : (INT16_MIN + 1024);
  void* __restrict__ H = D.H;
  void* __restrict__ F = D.F;
  void* __restrict__ O = D.O;
  void* __restrict__ E = D.E;
  void* __restrict__ Q = D.Q;
  const P NEG2 = Lx::splat(Lx::kNeg);
  const uint32_t NZ = S.min16x2;
  const P m2 = Lx::splat(m), n2 = Lx::splat(n);
  const P g2 = Lx::splat(g), e2 = Lx::splat(e), q2 = Lx::splat(q), c2 = Lx::splat(c);
  const P ge2 = Lx::splat(g - e), qc2 = Lx::splat(q - c);
  auto first_col = [&](uint32_t sg) { return (sg * nt + t) * CPT; };
  // row 0 (implementation.hpp:555-694)
  auto ramp = [&](int32_t j) -> int32_t {
    if (type == kSW) return 0;
    if (SUB == kConvex) return imax(g + j * e, q + j * c);
    if (SUB == kAffine) return g + j * e;
    return g + j * g;
  };
#pragma unroll 1
  for (int sg = 0; sg < SEGS; ++sg) {
    const uint32_t s0 = first_col(sg);
    const uint64_t w0 = 2 * (uint64_t)(sg * nt + t);
#pragma unroll
    for (int k = 0; k < HP; k += 2) {
      const P h0 = Lx::make(ramp((int32_t)(s0 + k)), ramp((int32_t)(s0 + HP + k)));
      const P h1 = Lx::make(ramp((int32_t)(s0 + k + 1)), ramp((int32_t)(s0 + HP + k + 1)));
      const uint64_t wk = w0 + (k / 2) * st2;
      Lx::store2(H, wk, h0, h1);
      if (SUB >= kAffine) Lx::store2(F, wk, NEG2, NEG2);
      if (SUB == kConvex) Lx::store2(O, wk, NEG2, NEG2);
    }
  }
  if (t == 0) {
    D.fc[0] = 0;
    D.fcF[0] = 0;
    D.fcO[0] = 0;
  }
  int32_t bval = type == kSW ? 0 : (type == kOV ? kNegBig : NEGW);
  int32_t brow = -1;
  int32_t first_sink = -1;
  // the strip holding column L-1 (NW selection)
  const uint32_t tv_last = (L - 1) / CPT;
  const int32_t last_k = (int32_t)(((L - 1) % CPT) % HP), last_hi = (int32_t)(((L - 1) % CPT) / HP);
  __syncthreads();
  for (uint32_t i = 1; i <= V; ++i) {
    const uint4 rec = D.rowrec[i];
    const uint32_t rflags = (rec.y >> 16) & 0xFFu;
    const L16::P rc2 = L16::splat(rec.y >> 24);
    const uint32_t pb = rec.x, pe = D.pred_ptr[i + 1];
    // first column (thread 0): NW takes the best predecessor's plus a gap
    int32_t fci = 0;
    if (t == 0) {
      int32_t fl = kNegBig, fa = kNegBig, fo = kNegBig;
      for (uint32_t pi = pb; pi < pe; ++pi) {
        const uint32_t p = D.preds[pi];
        fl = imax(fl, D.fc[p]);
        if (SUB >= kAffine) fa = imax(fa, D.fcF[p]);
        if (SUB == kConvex) fo = imax(fo, D.fcO[p]);
      }
      const bool source = (rflags & kRowSource) != 0;
      if (type == kNW) {
        if (SUB == kLinear) {
          fci = (source ? 0 : fl) + g;
        } else {
          const int32_t vF = (source ? g - e : fa) + e;
          D.fcF[i] = vF;
          if (SUB == kConvex) {
            const int32_t vO = (source ? q - c : fo) + c;
            D.fcO[i] = vO;
            fci = imax(vF, vO);
          } else {
            fci = vF;
          }
        }
      }
      D.fc[i] = fci;
    }
    // scan carries from the previous strip (thread 0)
    int32_t carry_q = 0, carry_e = 0, carry_h = 0;
#pragma unroll 1
    for (int sg = 0; sg < SEGS; ++sg) {
      const uint32_t tv = sg * nt + t;
      const uint32_t s0 = tv * CPT;
      const uint64_t w0 = 2 * (uint64_t)tv;
      uint32_t c8[(HP + 3) / 4], ch8[(HP + 3) / 4];
#pragma unroll
      for (int k4 = 0; k4 < (HP + 3) / 4; ++k4) {
        uint32_t lo = 0, hi = 0;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          const uint32_t k = k4 * 4 + b;
          const uint32_t jl = s0 + k, jh = s0 + HP + k;
          lo |= (k < HP && jl < L ? (uint32_t)seq[jl] : 0xFFu) << (8 * b);
          hi |= (k < HP && jh < L ? (uint32_t)seq[jh] : 0xFFu) << (8 * b);
        }
        c8[k4] = lo;
        ch8[k4] = hi;
      }
      // every predecessor, the previous row included, from memory
      P hd[HP], f[HP], o[HP];
      bool first = true;
      for (uint32_t pi = pb; pi < pe; ++pi) {
        const uint32_t p = D.preds[pi];
        P hp[HP], fp[HP], op[HP];
        const uint64_t rwp = (uint64_t)p * wrow + w0;
#pragma unroll
        for (int k = 0; k < HP; k += 2) {
          const uint64_t wk = rwp + (k / 2) * st2;
          Lx::load2(H, wk, hp[k], hp[k + 1]);
          if (SUB >= kAffine) Lx::load2(F, wk, fp[k], fp[k + 1]);
          if (SUB == kConvex) Lx::load2(O, wk, op[k], op[k + 1]);
        }
        const int32_t hleft = tv == 0 ? D.fc[p]
                                      : Lx::elem(H, (uint64_t)p * ld + 2 * ((HP / 2 - 1) * st2 + w0 - 1) + 1);
#pragma unroll
        for (int k = 0; k < HP; ++k) {
          const P left = k == 0 ? Lx::make(hleft, Lx::lo(hp[HP - 1])) : hp[k - 1];
          hd[k] = first ? left : Lx::max(hd[k], left, NZ);
          if (SUB == kLinear) {
            f[k] = first ? hp[k] : Lx::max(f[k], hp[k], NZ);
          } else {
            f[k] = first ? Lx::addmax(hp[k], ge2, fp[k]) : Lx::max3(f[k], Lx::add(hp[k], ge2), fp[k]);
            if (SUB == kConvex)
              o[k] = first ? Lx::addmax(hp[k], qc2, op[k]) : Lx::max3(o[k], Lx::add(hp[k], qc2), op[k]);
          }
        }
        first = false;
      }
      const uint64_t rw = (uint64_t)i * wrow + w0;
      P h[HP];
#pragma unroll
      for (int k = 0; k < HP; ++k) {
        const uint32_t chars = __byte_perm(c8[k / 4], ch8[k / 4], (uint32_t)(k % 4) | (0x4u + k % 4) << 8) &
                               0x00FF00FFu;
        const P d = Lx::add(hd[k], Lx::profile(chars, rc2.v, m2, n2));
        if (SUB == kLinear) {
          h[k] = Lx::addmax(f[k], g2, d);
        } else {
          f[k] = Lx::add(f[k], e2);
          if (SUB == kConvex) {
            o[k] = Lx::add(o[k], c2);
            h[k] = Lx::max3(d, f[k], o[k]);
          } else {
            h[k] = Lx::max(d, f[k], NZ);
          }
        }
      }
      if (SUB >= kAffine) {
#pragma unroll
        for (int k = 0; k < HP; k += 2) {
          Lx::store2(F, rw + (k / 2) * st2, f[k], f[k + 1]);
          if (SUB == kConvex) Lx::store2(O, rw + (k / 2) * st2, o[k], o[k + 1]);
        }
      }
      P hs[HP], ee[HP], qq[HP];
      int32_t out_q = 0, out_e = 0, out_h = 0;  // this strip's carries (its last column)
      if (SUB == kLinear) {
#pragma unroll
        for (int k = 0; k < HP; ++k) hs[k] = h[k];
        pair_scan<CPT, Lx>(hs, sg == 0 ? fci : carry_h, g, sh.wv);
        out_h = Lx::hi(hs[HP - 1]);
        if (type == kSW) {
          const P z = Lx::splat(0);
#pragma unroll
          for (int k = 0; k < HP; ++k) hs[k] = Lx::max(hs[k], z, NZ);
        }
      } else {
        if (SUB == kConvex) {
          P x[HP];
#pragma unroll
          for (int k = 0; k < HP; ++k) x[k] = Lx::add(h[k], q2);
          const int32_t qin = pair_scan<CPT, Lx>(x, sg == 0 ? fci + q : carry_q, c, sh.wq);
          out_q = Lx::hi(x[HP - 1]);
          qq[0] = Lx::make(qin, Lx::lo(x[HP - 1]));
#pragma unroll
          for (int k = 1; k < HP; ++k) qq[k] = x[k - 1];
        }
        {
          uint32_t bmap = 0;
          if (SUB == kConvex) {
#pragma unroll
            for (int k = 0; k < HP; ++k) {
              if ((s0 + k + 1) % (uint32_t)lanes == 0) bmap |= 1u << k;
              if ((s0 + HP + k + 1) % (uint32_t)lanes == 0) bmap |= 1u << (16 + k);
            }
          }
          P x[HP];
#pragma unroll
          for (int k = 0; k < HP; ++k) {
            if (SUB == kConvex) {
              const uint32_t bm = sign_lanes(bmap << (15 - k));
              x[k] = Lx::add(Lx::max(h[k], Lx::select(bm, qq[k], NEG2), NZ), g2);
            } else {
              x[k] = Lx::add(h[k], g2);
            }
          }
          const int32_t ein = pair_scan<CPT, Lx>(x, sg == 0 ? fci + g : carry_e, e, sh.wv);
          out_e = Lx::hi(x[HP - 1]);
          ee[0] = Lx::make(ein, Lx::lo(x[HP - 1]));
#pragma unroll
          for (int k = 1; k < HP; ++k) ee[k] = x[k - 1];
        }
#pragma unroll
        for (int k = 0; k < HP; ++k) {
          if (SUB == kConvex)
            hs[k] = type == kSW ? Lx::max3_relu(h[k], ee[k], qq[k]) : Lx::max3(h[k], ee[k], qq[k]);
          else
            hs[k] = type == kSW ? Lx::max3_relu(h[k], ee[k], ee[k]) : Lx::max(h[k], ee[k], NZ);
        }
      }
      if (SUB >= kAffine) {
#pragma unroll
        for (int k = 0; k < HP; k += 2) {
          Lx::store2cs(E, rw + (k / 2) * st2, ee[k], ee[k + 1]);
          if (SUB == kConvex) Lx::store2cs(Q, rw + (k / 2) * st2, qq[k], qq[k + 1]);
        }
      }
#pragma unroll
      for (int k = 0; k < HP; k += 2) Lx::store2(H, rw + (k / 2) * st2, hs[k], hs[k + 1]);
      // row selection (strict <: the earliest row wins a tie)
      if (type == kNW) {
        if ((rflags & kRowSink) && tv == tv_last) {
          int32_t v = kNegBig;
#pragma unroll
          for (int k = 0; k < HP; ++k)
            if (k == last_k) v = last_hi ? Lx::hi(hs[k]) : Lx::lo(hs[k]);
          if (v > bval) {
            bval = v;
            brow = (int32_t)i;
          }
        }
      } else if ((type == kSW || (rflags & kRowSink)) && s0 < L) {
        P mx = NEG2;
#pragma unroll
        for (int k = 0; k < HP; ++k) {
          const uint32_t vm = (s0 + k < L ? 0x0000FFFFu : 0u) | (s0 + HP + k < L ? 0xFFFF0000u : 0u);
          mx = Lx::max(mx, Lx::select(vm, hs[k], NEG2), NZ);
        }
        const int32_t tm = imax(Lx::lo(mx), Lx::hi(mx));
        if (tm > bval) {
          bval = tm;
          brow = (int32_t)i;
        }
      }
      // hand this strip's carries to thread 0 for the next strip
      if (SEGS > 1 && sg + 1 < SEGS) {
        if (t == nt - 1) {
          sh.bcast[0] = out_q;
          sh.bcast[1] = out_e;
          sh.bcast[2] = out_h;
        }
        __syncthreads();
        carry_q = sh.bcast[0];
        carry_e = sh.bcast[1];
        carry_h = sh.bcast[2];
        __syncthreads();
      }
    }
    if (type == kOV && (rflags & kRowSink) && first_sink < 0) first_sink = (int32_t)i;
    __syncthreads();
  }

  // global selection: best value, then the earliest row reaching it
  const int32_t B = block_max(bval, sh);
  const int32_t R = block_min(bval == B && brow >= 0 ? brow : 0x7fffffff, sh);
  int64_t max_i = -1;
  int32_t score = 0;
  if (type == kSW) {
    if (B > 0 && R != 0x7fffffff) {
      max_i = R;
      score = B;
    }
  } else if (type == kOV) {
    if (B > 0) {
      max_i = R;
      score = B;
    } else {
      max_i = first_sink;
      score = 0;
    }
  } else {
    if (R != 0x7fffffff && B > NEGW) {
      max_i = R;
      score = B;
    }
  }
  int64_t max_j = -1;
  if (max_i >= 0) {
    if (type == kNW) {
      max_j = (int64_t)L - 1;
    } else {
      const uint64_t base = (uint64_t)max_i * ld;
      int32_t jj = 0x7fffffff;
      for (int sg = 0; sg < SEGS && jj == 0x7fffffff; ++sg)
        for (int r = 0; r < CPT && jj == 0x7fffffff; ++r) {
          const uint32_t j = first_col(sg) + r;
          if (j < L && Lx::elem(H, base + colmap<CPT>(j, ntv)) == score) jj = (int32_t)j;
        }
      jj = block_min(jj, sh);
      max_j = jj == 0x7fffffff ? -1 : jj;
    }
  }
  *out_max_i = max_i;
  *out_max_j = max_j;
  *out_score = score;
}
// Traceback from (max_i, max_j) (implementation.hpp:955-1124, 1324-1574,
// 1826-2121), thread 0.  Every move is re-derived from the stored
// H/F/O/E/Q rows with the reference's tests in the reference's order.
// Pairs are written to `out` in forward order.
template <int SUB, int CPT, typename T>
static __device__ __noinline__ int32_t dp_traceback(const Scoring& S, const DpView& D, const GraphView& G,
                                const uint8_t* seq, uint32_t L, uint32_t V, int64_t max_i,
                                int64_t max_j, int32_t* out, uint32_t* n_out, uint32_t ntv) {
  using Lx = Lanes<T>;
  const uint64_t ld = D.caps.ld;
  const int32_t type = S.type;
  const int32_t m = S.m, n = S.n, g = S.g, e = S.e, q = S.q, c = S.c;
  const void* H = D.H;
  const void* F = D.F;
  const void* O = D.O;
  const void* E = D.E;
  const void* Q = D.Q;
  const uint64_t nt = ntv;  // the forward pass's row width in strips
  auto at = [&](const void* M, int64_t row, int64_t col) -> int32_t {
    return Lx::elem(M, (uint64_t)row * ld + colmap<CPT>((uint64_t)col, nt));
  };
  // H, E or Q of column col, where column -1 is the first column: the
  // forward pass starts all three in-row recurrences from it
  auto left = [&](const void* M, int64_t row, int64_t col) -> int32_t {
    return col < 0 ? D.fc[row] : at(M, row, col);
  };
  // extend_left continues past column cc (implementation.hpp:2031-2035):
  // E (and Q, convex) of cc extend the values of column cc-1
  auto run = [&](int64_t row, int64_t cc) -> bool {
    bool r = at(E, row, cc) == left(E, row, cc - 1) + e;
    if (SUB == kConvex) r = r && at(Q, row, cc) == left(Q, row, cc - 1) + c;
    return r;
  };
  int32_t* tb = out;  // written back to front, reversed at the end
  uint64_t np = 0;
  const uint64_t cap = D.aln_cap;
  int64_t i = max_i, j = max_j, prev_i = 0, prev_j = 0;
  uint64_t guard = 0;
  const uint64_t guard_max = 4 * ((uint64_t)V + L) + 64;
#define EMIT(a, b)                    \
  do {                                \
    if (np >= cap) return kTraceback; \
    tb[2 * np] = (a);                 \
    tb[2 * np + 1] = (b);             \
    ++np;                             \
  } while (0)
  // The path mostly steps diagonally through the previous ranks: the H
  // cells kTbAhead steps ahead on the current diagonal and on the diagonal
  // one row up (where it continues after a vertical move) are prefetched
  // into L1 while this step is tested, so the walk rarely waits for DRAM.
  constexpr int64_t kTbAhead = 8;
  auto prefetch = [&](int64_t row, int64_t col) {
#ifdef __CUDA_ARCH__
    const char* p = static_cast<const char*>(H) +
                    sizeof(T) * ((uint64_t)row * ld + colmap<CPT>((uint64_t)col, nt));
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
#else
    (void)row;
    (void)col;
#endif
  };
  while (true) {
    if (++guard > guard_max) return kTraceback;
    if (j == -1 || i == 0) break;
    if (i > kTbAhead + 1 && j >= kTbAhead) {
      prefetch(i - kTbAhead, j - kTbAhead);
      prefetch(i - kTbAhead - 1, j - kTbAhead);
    }
    const uint32_t node = G.rank_to_node[i - 1];
    const int32_t h = at(H, i, j);
    if (type == kSW && h == 0) break;
    const uint32_t pb = D.pred_ptr[i], pe = D.pred_ptr[i + 1];
    const int32_t prf = D.row_char[i] == seq[j] ? m : n;
    bool found = false, ext_left = false, ext_up = false;
    for (uint32_t pi = pb; pi < pe; ++pi) {
      const int64_t p = D.preds[pi];
      const int32_t hd = j ? at(H, p, j - 1) : D.fc[p];
      if (h == hd + prf) {
        prev_i = p;
        prev_j = j - 1;
        found = true;
        break;
      }
    }
    if (!found) {
      for (uint32_t pi = pb; pi < pe; ++pi) {
        const int64_t p = D.preds[pi];
        const int32_t hp = at(H, p, j);
        bool take;
        if (SUB == kLinear) {
          take = h == hp + g;
        } else if (SUB == kAffine) {
          ext_up = h == at(F, p, j) + e;
          take = ext_up || h == hp + g;
        } else {
          ext_up = h == at(F, p, j) + e;
          if (ext_up) {
            take = true;
          } else if (h == hp + g) {
            take = true;
          } else {
            ext_up = h == at(O, p, j) + c;
            take = ext_up || h == hp + q;
          }
        }
        if (take) {
          prev_i = p;
          prev_j = j;
          found = true;
          break;
        }
      }
    }
    if (!found) {
      // horizontal tests in the reference's order (implementation.hpp
      // 1977-1990): E extension, H + g, Q extension, H + q
      const int32_t hl = left(H, i, j - 1);
      bool any;
      if (SUB == kLinear) {
        any = h == hl + g;
      } else {
        const bool mA = h == left(E, i, j - 1) + e;
        const bool mB = h == hl + g;
        any = mA || mB;
        ext_left = mA;
        if (SUB == kConvex && !any) {
          const bool mC = h == left(Q, i, j - 1) + c;
          any = mC || h == hl + q;
          ext_left = mC;
        }
      }
      if (any) {
        prev_i = i;
        prev_j = j - 1;
        found = true;
      }
    }
    EMIT(i == prev_i ? -1 : (int32_t)node, j == prev_j ? -1 : (int32_t)j);
    i = prev_i;
    j = prev_j;
    if (SUB >= kAffine && ext_left) {
      while (true) {
        if (++guard > guard_max) return kTraceback;
        EMIT(-1, (int32_t)j);
        --j;
        if (j == -1) break;
        if (!run(i, j + 1)) break;
      }
    } else if (SUB >= kAffine && ext_up) {
      while (true) {
        if (++guard > guard_max) return kTraceback;
        const uint32_t un = G.rank_to_node[i - 1];
        const int32_t fv = at(F, i, j);
        const uint32_t pb2 = D.pred_ptr[i];
        const uint32_t pe2 = D.row_indeg[i] ? D.pred_ptr[i + 1] : pb2;  // sources: none
        bool stop;
        prev_i = 0;
        if (SUB == kAffine) {
          stop = false;
          for (uint32_t pi = pb2; pi < pe2; ++pi) {
            const int64_t p = D.preds[pi];
            stop = fv == at(H, p, j) + g;
            if (stop || fv == at(F, p, j) + e) {
              prev_i = p;
              break;
            }
          }
        } else {
          const int32_t ov = at(O, i, j);
          stop = true;
          for (uint32_t pi = pb2; pi < pe2; ++pi) {
            const int64_t p = D.preds[pi];
            if (fv == at(F, p, j) + e || ov == at(O, p, j) + c) {
              prev_i = p;
              stop = false;
              break;
            }
          }
          if (stop) {
            for (uint32_t pi = pb2; pi < pe2; ++pi) {
              const int64_t p = D.preds[pi];
              const int32_t hp = at(H, p, j);
              if (fv == hp + g || ov == hp + q) {
                prev_i = p;
                break;
              }
            }
          }
        }
        EMIT((int32_t)un, -1);
        i = prev_i;
        if (stop || i == 0) break;
      }
    }
  }
  if (type == kNW) {
    while (i == 0 && j != -1) {
      EMIT(-1, (int32_t)j);
      --j;
    }
    while (i != 0 && j == -1) {
      if (++guard > guard_max) return kTraceback;
      const uint32_t un = G.rank_to_node[i - 1];
      EMIT((int32_t)un, -1);
      if (D.row_indeg[i] == 0) {
        i = 0;
      } else {
        for (uint32_t pi = D.pred_ptr[i]; pi < D.pred_ptr[i + 1]; ++pi) {
          const int64_t p = D.preds[pi];
          bool hit;
          if (SUB == kLinear) {
            hit = D.fc[i] == D.fc[p] + g;
          } else if (SUB == kAffine) {
            hit = D.fcF[i] == D.fcF[p] + e;
          } else {
            hit = D.fcF[i] == D.fcF[p] + e || D.fcO[i] == D.fcO[p] + c;
          }
          if (hit) {
            i = p;
            break;
          }
        }
      }
    }
  }
#undef EMIT
  for (uint64_t a = 0, b = np ? np - 1 : 0; a < b; ++a, --b) {
    const int32_t x0 = tb[2 * a], x1 = tb[2 * a + 1];
    tb[2 * a] = tb[2 * b];
    tb[2 * a + 1] = tb[2 * b + 1];
    tb[2 * b] = x0;
    tb[2 * b + 1] = x1;
  }
  *n_out = (uint32_t)np;
  return kOk;
}

}  // namespace spoa_gb300
