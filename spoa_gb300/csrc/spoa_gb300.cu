// spoa_gb300.cu - host side and C ABI of the GB300 POA library.
// The kernel templates are in poa_kernels.cuh.
//
// Kernels (one CTA owns one window; see poa_device.cuh / poa_dp.cuh):
//   k_graph_reset       empty graph (Graph::Graph, Graph::Clear)
//   k_align<SUB,CPT>    one read against a graph (AlignmentEngine::Align)
//   k_add               Graph::AddAlignment + TopologicalSort
//   k_align_add<..>     fused per-read body of spoa's CLI loop
//   k_consensus         Graph::GenerateConsensus
//   k_msa               Graph::GenerateMultipleSequenceAlignment
//   k_export            flat copy for the host-side node/edge views
//   k_batch<SUB,CPT>    persistent kernel: CTAs pull whole windows from a
//                       device work queue and run every read of the window,
//                       then the consensus (and optionally the MSA)
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <deque>
#include <vector>

#include "../../include/spoa_gb300.h"
#include "gfa_text.h"
#define SPOA_GB300_HOST_TU
#include "poa_kernels.cuh"

namespace spoa_gb300 {
#define SPOA_EXTERN(SUB, T)                                                                      \
  extern template int32_t launch_align<SUB, T>(int, int, const Scoring&, const GraphView&,      \
                                               const DpView&, const uint8_t*, uint32_t,         \
                                               ReadOut*);                                       \
  extern template int32_t launch_align_add<SUB, T>(int, int, const Scoring&, const GraphView&,  \
                                                   const DpView&, const uint8_t*, uint32_t,     \
                                                   const uint8_t*, int32_t, ReadOut*,           \
                                                   const ReadOut*, cudaStream_t);               \
  extern template int32_t launch_batch<SUB, T>(int, int, int, const BatchArgs&, cudaStream_t);  \
  extern template int32_t occupancy_batch<SUB, T>(int, int, int*);                               \
  extern template int32_t launch_serve<SUB, T>(int, int, int, const ServeArgs&, cudaStream_t);  \
  extern template int32_t occupancy_serve<SUB, T>(int, int, int*);
SPOA_EXTERN(kLinear, int16_t)
SPOA_EXTERN(kAffine, int16_t)
SPOA_EXTERN(kConvex, int16_t)
SPOA_EXTERN(kLinear, int32_t)
SPOA_EXTERN(kAffine, int32_t)
SPOA_EXTERN(kConvex, int32_t)
#undef SPOA_EXTERN
#define SPOA_EXTERN_SEG(SUB)                                                                     \
  extern template int32_t launch_batch_seg<SUB, int32_t>(int, int, int, const BatchArgs&,        \
                                                         cudaStream_t);                          \
  extern template int32_t occupancy_batch_seg<SUB, int32_t>(int, int, int*);                     \
  extern template int32_t launch_batch_cl<SUB>(int, int, int, const BatchArgs&, cudaStream_t);   \
  extern template int32_t occupancy_batch_cl<SUB>(int, int, int*);
SPOA_EXTERN_SEG(kLinear)
SPOA_EXTERN_SEG(kAffine)
SPOA_EXTERN_SEG(kConvex)
#undef SPOA_EXTERN_SEG
#define SPOA_EXTERN_MW(SUB)                                                                      \
  extern template int32_t launch_batch_mw<SUB>(int, int, int, int, const BatchArgs&,             \
                                               cudaStream_t);                                    \
  extern template int32_t occupancy_batch_mw<SUB>(int, int, int, int*);                         \
  extern template int32_t launch_batch_r128<SUB>(int, int, const BatchArgs&, cudaStream_t);     \
  extern template int32_t occupancy_batch_r128<SUB>(int, int*);
SPOA_EXTERN_MW(kLinear)
SPOA_EXTERN_MW(kAffine)
SPOA_EXTERN_MW(kConvex)
#undef SPOA_EXTERN_MW
}  // namespace spoa_gb300

// ===========================================================================
// host side
// ===========================================================================
using namespace spoa_gb300;

namespace {

constexpr int kCpts16[] = {8, 12, 16, 20, 24, 32};
constexpr int kCpts32[] = {8, 12, 16, 24, 32};

#define CU(call)                                \
  do {                                          \
    cudaError_t err__ = (call);                 \
    if (err__ != cudaSuccess) return kCuda;     \
  } while (0)

// fn<gap model, lane type>(...) for a runtime gap model and width
#define SPOA_BY_SUB(sub, wide, fn, ...)                                                  \
  ((wide) ? ((sub) == kLinear   ? fn<kLinear, int32_t>(__VA_ARGS__)                      \
             : (sub) == kAffine ? fn<kAffine, int32_t>(__VA_ARGS__)                      \
             : (sub) == kConvex ? fn<kConvex, int32_t>(__VA_ARGS__)                      \
                                : (int32_t)kInvalidArgument)                             \
          : ((sub) == kLinear   ? fn<kLinear, int16_t>(__VA_ARGS__)                      \
             : (sub) == kAffine ? fn<kAffine, int16_t>(__VA_ARGS__)                      \
             : (sub) == kConvex ? fn<kConvex, int16_t>(__VA_ARGS__)                      \
                                : (int32_t)kInvalidArgument))

// fn<gap model, int32_t>(...) for the kernels built for 32-bit lanes only
#define SPOA_BY_SUB32(sub, fn, ...)                                                      \
  ((sub) == kLinear   ? fn<kLinear, int32_t>(__VA_ARGS__)                                \
   : (sub) == kAffine ? fn<kAffine, int32_t>(__VA_ARGS__)                                \
   : (sub) == kConvex ? fn<kConvex, int32_t>(__VA_ARGS__)                                \
                      : (int32_t)kInvalidArgument)

// fn<gap model>(...) for the kernels built for 16-bit lanes only
#define SPOA_BY_SUB16(sub, fn, ...)                                                      \
  ((sub) == kLinear   ? fn<kLinear>(__VA_ARGS__)                                         \
   : (sub) == kAffine ? fn<kAffine>(__VA_ARGS__)                                         \
   : (sub) == kConvex ? fn<kConvex>(__VA_ARGS__)                                         \
                      : (int32_t)kInvalidArgument)

// 32-bit rows wider than this run on thread-block clusters (k_batch_cl).
constexpr uint32_t kClusterMinCols = 1536;

// Latency tile: the smallest strip (most threads) that covers L.
bool latency_tile(uint32_t L, bool wide, int* cpt, int* nt) {
  const int* cs = wide ? kCpts32 : kCpts16;
  const int nc = wide ? 5 : 6;
  for (int k = 0; k < nc; ++k) {
    const int c = cs[k];
    uint64_t t = ((uint64_t)(L + c - 1) / c + 31) / 32 * 32;
    if (t == 0) t = 32;
    if (t <= 1024) {
      *cpt = c;
      *nt = (int)t;
      return true;
    }
  }
  return false;
}

// Throughput tile: fewest padded columns, then fewest threads.
bool throughput_tile(uint32_t L, bool wide, int* cpt, int* nt) {
  uint64_t best = ~0ull;
  const int* cs = wide ? kCpts32 : kCpts16;
  const int nc = wide ? 5 : 6;
  for (int k = 0; k < nc; ++k) {
    const int c = cs[k];
    uint64_t t = ((uint64_t)(L + c - 1) / c + 31) / 32 * 32;
    if (t == 0) t = 32;
    if (t > 512) continue;  // 512 threads x 128 registers fill the register file
    uint64_t cost = t * (uint64_t)c;
    if (cost < best || (cost == best && (int)t < *nt)) {
      best = cost;
      *cpt = c;
      *nt = (int)t;
    }
  }
  return best != ~0ull;
}

// Segmented tile for 32-bit rows wider than one 12-column strip per thread
// covers (12 x 512): strips of 12 columns, the fewest strips per thread (2,
// 4 or 8) that keep the CTA at 512 threads or fewer.  Each thread then holds
// 12 columns in registers at a time instead of 16-32, which spill.
bool seg_tile(uint32_t L, int* cpt, int* nt, int* segs) {
  for (int s = 2; s <= 8; s *= 2) {
    const uint64_t per = (uint64_t)kSegCpt * s;
    const uint64_t t = std::max<uint64_t>(32, ((uint64_t)(L + per - 1) / per + 31) / 32 * 32);
    if (t <= 512) {
      *cpt = kSegCpt;
      *nt = (int)t;
      *segs = s;
      return true;
    }
  }
  return false;
}

// Cluster tile for `windows` windows of 32-bit rows of up to L columns
// (wider than kClusterMinCols): 2, 4 or 8 CTAs per window, 12 columns per
// thread, the fewest 32-thread multiples per CTA that cover L.  The
// smallest cluster that holds the row, doubled while the windows' clusters
// still fit one CTA per SM: a lone window runs fastest on the most SMs (the
// 10-kb window: 3.23 s on 8 CTAs, 3.56 s on 4, 4.42 s on 2), a batch of
// many on the fewest per window (2,000 uneven windows: 111.8 windows/s on
// 2 CTAs, 93.3 on 4).  `force` (2, 4 or 8) asks for that many CTAs, or
// more when the row needs them.  False when L is not in the clusters' range
// (up to 8 x 512 x 12 columns).
bool cluster_tile(uint32_t L, uint64_t windows, int sm_count, int force, int* cl, int* nt) {
  if (L <= kClusterMinCols || L > (uint32_t)kClCpt * 8 * 512) return false;
  int c = L > 4u * 512 * kClCpt ? 8 : L > 2u * 512 * kClCpt ? 4 : 2;
  if (force == 2 || force == 4 || force == 8)
    c = std::max(c, force);
  else
    while (c < 8 && std::max<uint64_t>(windows, 1) * (uint64_t)(2 * c) <= (uint64_t)sm_count)
      c *= 2;
  const uint64_t per = (uint64_t)c * kClCpt;
  *cl = c;
  *nt = (int)std::max<uint64_t>(32, ((L + per - 1) / per + 31) / 32 * 32);
  return true;
}

// Makes `dev` the calling thread's current device while the guard lives and
// restores the previous current device afterwards.
struct DeviceGuard {
  int prev = -1;
  bool ok = true;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) {
      cudaGetLastError();
      prev = -1;
      ok = false;
      return;
    }
    if (prev != dev && cudaSetDevice(dev) != cudaSuccess) {
      cudaGetLastError();
      ok = false;
    }
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

// The device a batch or server runs on: the requested ordinal, or the
// calling thread's current device; -1 when the ordinal does not exist.
int resolve_device(int32_t set, int32_t ordinal) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  if (set) return ordinal >= 0 && ordinal < n ? ordinal : -1;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  return dev;
}

struct DeviceBuf {
  void* p = nullptr;
  size_t n = 0;
  ~DeviceBuf() { if (p) cudaFree(p); }
  int32_t ensure(size_t bytes) {
    if (bytes <= n) return kOk;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    if (cudaMalloc(&p, bytes ? bytes : 1) != cudaSuccess) {
      cudaGetLastError();
      return kNoMemory;
    }
    n = bytes;
    return kOk;
  }
  template <typename T> T* as() const { return static_cast<T*>(p); }
};

}  // namespace

struct spoa_gb300_engine {
  Scoring S;
  DeviceBuf dp_arena;
  DpView dv{};
  DpCaps dcaps{};
  DeviceBuf seq, qual, out;
  ReadOut* h_out = nullptr;
  int device = 0;
  uint32_t pre_rows = 0, pre_ld = 0;
};

struct spoa_gb300_graph {
  DeviceBuf arena;
  GraphView v{};
  GraphCaps caps{};
  GraphHeader h{};  // host copy of the header, refreshed after each change
  DeviceBuf seq, w, pairs, stat;
  int device = 0;
};

namespace {

int32_t graph_refresh(spoa_gb300_graph* g) {
  CU(cudaMemcpy(&g->h, g->v.hdr, sizeof(GraphHeader), cudaMemcpyDeviceToHost));
  return kOk;
}

// Grows the graph arena so that `len` more bases fit; contents are kept.
int32_t graph_reserve(spoa_gb300_graph* g, uint64_t len, uint64_t reads = 1) {
  const GraphHeader& h = g->h;
  GraphCaps need = g->caps;
  auto grow = [](uint32_t cap, uint64_t want) {
    uint64_t c = cap ? cap : 256;
    while (c < want) c *= 2;
    return (uint32_t)std::min<uint64_t>(c, 0xFFFFFFF0u);
  };
  need.nodes = grow(g->caps.nodes, (uint64_t)h.n_nodes + len + 1);
  need.edges = grow(g->caps.edges, (uint64_t)h.n_edges + len + reads + 1);
  need.labels = grow(g->caps.labels, (uint64_t)h.n_labels + len + reads + 1);
  need.seqs = grow(g->caps.seqs, (uint64_t)h.n_seqs + reads + 1);
  if (g->arena.p && need.nodes == g->caps.nodes && need.edges == g->caps.edges &&
      need.labels == g->caps.labels && need.seqs == g->caps.seqs)
    return kOk;
  GraphView nv;
  uint64_t bytes = graph_layout(nullptr, need, &nv);
  DeviceBuf fresh;
  if (fresh.ensure(bytes)) return kNoMemory;
  graph_layout(fresh.as<uint8_t>(), need, &nv);
  if (g->arena.p) {
    const GraphView& o = g->v;
    const uint64_t N = h.n_nodes, E = h.n_edges, Lb = h.n_labels, Sq = h.n_seqs;
    const uint32_t K = need.aligned;
    CU(cudaMemcpy(nv.hdr, o.hdr, sizeof(GraphHeader), cudaMemcpyDeviceToDevice));
#define CP(field, count, esz) \
  if ((count) != 0) CU(cudaMemcpy(nv.field, o.field, (count) * (esz), cudaMemcpyDeviceToDevice))
    CP(code, N, 1);
    CP(nlink, N, 16);
    CP(in_deg, N, 4);
    CP(n_aligned, N, 1);
    CP(aligned, N * K, 4);
    CP(nrec, N, 16);
    CP(rank_to_node, N, 4);
    CP(node_to_rank, N, 4);
    CP(erec, E, 16);
    CP(e_lab_first, E, 4);
    CP(e_lab_last, E, 4);
    CP(e_weight, E, 8);
    CP(lab_seq, Lb, 4);
    CP(lab_next, Lb, 4);
    CP(seq_begin, Sq, 4);
    CP(consensus, N, 4);
#undef CP
  } else {
    k_graph_reset<<<1, 32>>>(nv);
    CU(cudaGetLastError());
  }
  std::swap(g->arena.p, fresh.p);
  std::swap(g->arena.n, fresh.n);
  g->v = nv;
  g->caps = need;
  return kOk;
}

int32_t engine_reserve(spoa_gb300_engine* en, uint32_t rows, uint32_t ld, uint32_t preds) {
  DpCaps c = en->dcaps;
  bool grow = !en->dp_arena.p || rows > c.rows || ld > c.ld || preds > c.preds;
  if (!grow) return kOk;
  c.rows = std::max(rows, c.rows);
  c.ld = std::max(ld, c.ld);
  c.preds = std::max(preds, c.preds);
  c.sub = en->S.sub;
  DpView v;
  uint64_t bytes = dp_layout(nullptr, c, &v);
  en->dp_arena.~DeviceBuf();
  new (&en->dp_arena) DeviceBuf();
  if (en->dp_arena.ensure(bytes)) {
    en->dcaps = DpCaps{};
    return kNoMemory;
  }
  dp_layout(en->dp_arena.as<uint8_t>(), c, &v);
  en->dv = v;
  en->dcaps = c;
  return kOk;
}



int32_t prepare_read(spoa_gb300_engine* en, const spoa_gb300_graph* g, uint32_t L, bool wide,
                     int* cpt, int* nt) {
  if (!latency_tile(L, wide, cpt, nt)) return kTooLarge;
  int32_t st = engine_reserve(en, g->h.n_nodes + 1, (uint32_t)(*cpt) * (*nt),
                              g->h.n_edges + g->h.n_nodes + 2);
  if (st) return st;
  if (en->seq.ensure(std::max<size_t>(L, 1))) return kNoMemory;
  if (en->out.ensure(sizeof(ReadOut))) return kNoMemory;
  return kOk;
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

const char* spoa_gb300_status_string(int32_t s) {
  switch (s) {
    case kOk: return "ok";
    case kInvalidArgument: return "invalid argument";
    case kTooLarge: return "too large sequence!";
    case kOverflow: return "possible overflow!";
    case kNoMemory: return "insufficient memory!";
    case kInvalidAlignment: return "invalid alignment";
    case kMissingSequence: return "missing sequence in alignment";
    case kUnequalWeights: return "sequence and weights are of unequal size!";
    case kCapacity: return "device arena capacity exceeded";
    case kTraceback: return "traceback did not terminate";
    case kCuda: return "CUDA error";
    case SPOA_GB300_ERR_NEEDS_INT32: return "a read needs 32-bit scores";
    case SPOA_GB300_ERR_TIMEOUT: return "timed out";
    default: return "unknown status";
  }
}

int32_t spoa_gb300_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

int32_t spoa_gb300_engine_create(int32_t type, int8_t m, int8_t n, int8_t g, int8_t e,
                                 int8_t q, int8_t c, spoa_gb300_engine** out) {
  if (!out) return kInvalidArgument;
  *out = nullptr;
  if (type != kSW && type != kNW && type != kOV) return kInvalidArgument;
  if (g > 0 || q > 0) return kInvalidArgument;
  if (e > 0 || c > 0) return kInvalidArgument;
  int32_t sub = g >= e ? kLinear : ((g <= q || e >= c) ? kAffine : kConvex);
  if (sub == kLinear) {
    e = g;
  } else if (sub == kAffine) {
    q = g;
    c = e;
  }
  if (spoa_gb300_device_count() <= 0) return kCuda;
  auto* en = new (std::nothrow) spoa_gb300_engine();
  if (!en) return kNoMemory;
  en->S = Scoring{type, sub, m, n, g, e, q, c};
  cudaGetDevice(&en->device);
  if (cudaMallocHost(&en->h_out, sizeof(ReadOut)) != cudaSuccess) {
    cudaGetLastError();
    delete en;
    return kNoMemory;
  }
  *out = en;
  return kOk;
}

void spoa_gb300_engine_destroy(spoa_gb300_engine* en) {
  if (!en) return;
  if (en->h_out) cudaFreeHost(en->h_out);
  delete en;
}

int32_t spoa_gb300_engine_params(const spoa_gb300_engine* en, int32_t* type, int32_t* subtype,
                                 int8_t* p) {
  if (!en) return kInvalidArgument;
  if (type) *type = en->S.type;
  if (subtype) *subtype = en->S.sub;
  if (p) {
    p[0] = (int8_t)en->S.m; p[1] = (int8_t)en->S.n; p[2] = (int8_t)en->S.g;
    p[3] = (int8_t)en->S.e; p[4] = (int8_t)en->S.q; p[5] = (int8_t)en->S.c;
  }
  return kOk;
}

int32_t spoa_gb300_engine_prealloc(spoa_gb300_engine* en, uint32_t max_len, uint8_t alphabet) {
  if (!en) return kInvalidArgument;
  if (max_len > (uint32_t)INT32_MAX) return kTooLarge;
  // same early return as the reference: nothing to size when even int32
  // could overflow (implementation.hpp:392-397)
  int64_t wc = worst_case(en->S, (int64_t)max_len + 8, (int64_t)max_len * alphabet);
  if (wc < (int64_t)INT32_MIN + 1024) return kOk;
  int cpt, nt;
  if (!latency_tile(std::max<uint32_t>(max_len, 1), true, &cpt, &nt) &&
      !latency_tile(std::max<uint32_t>(max_len, 1), false, &cpt, &nt))
    return kNoMemory;
  uint64_t rows = (uint64_t)max_len * alphabet + 1;
  if (rows > 0xFFFFFFF0ull) return kNoMemory;
  DpCaps c{(uint32_t)rows, (uint32_t)(cpt * nt), (uint32_t)std::min<uint64_t>(3 * rows, 0xFFFFFFF0ull),
           en->S.sub};
  DpView v;
  uint64_t bytes = dp_layout(nullptr, c, &v);
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return kCuda;
  if (bytes > free_b) return kNoMemory;
  return engine_reserve(en, c.rows, c.ld, c.preds);
}

int32_t spoa_gb300_graph_create(spoa_gb300_graph** out) {
  if (!out) return kInvalidArgument;
  *out = nullptr;
  if (spoa_gb300_device_count() <= 0) return kCuda;
  auto* g = new (std::nothrow) spoa_gb300_graph();
  if (!g) return kNoMemory;
  cudaGetDevice(&g->device);
  g->caps = GraphCaps{0, 0, 0, 0, 31};
  std::memset(&g->h, 0, sizeof(g->h));
  int32_t st = graph_reserve(g, 1024);
  if (st == kOk) st = g->stat.ensure(16);
  if (st == kOk) st = graph_refresh(g);
  if (st != kOk) {
    delete g;
    return st;
  }
  *out = g;
  return kOk;
}

void spoa_gb300_graph_destroy(spoa_gb300_graph* g) { delete g; }

int32_t spoa_gb300_graph_clear(spoa_gb300_graph* g) {
  if (!g) return kInvalidArgument;
  k_graph_reset<<<1, 32>>>(g->v);
  CU(cudaGetLastError());
  return graph_refresh(g);
}

int32_t spoa_gb300_engine_align(spoa_gb300_engine* en, const char* seq, uint32_t L,
                                const spoa_gb300_graph* g, int32_t* score,
                                int32_t* score_written, int32_t* pairs, uint32_t pairs_cap,
                                uint32_t* n_pairs) {
  if (!en || !g || !n_pairs) return kInvalidArgument;
  *n_pairs = 0;
  if (score_written) *score_written = 0;
  if (L > (uint32_t)INT32_MAX) return kTooLarge;
  if (g->h.n_nodes == 0 || L == 0) return kOk;
  const int32_t lanes = lanes_for(en->S, L, g->h.n_nodes);
  if (!lanes) return kOverflow;
  const bool wide = lanes == 8;
  int cpt, nt;
  int32_t st = prepare_read(en, g, L, wide, &cpt, &nt);
  if (st) return st;
  CU(cudaMemcpy(en->seq.p, seq, L, cudaMemcpyHostToDevice));
  st = SPOA_BY_SUB(en->S.sub, wide, launch_align, cpt, nt, en->S, g->v, en->dv,
                   en->seq.as<uint8_t>(), L, en->out.as<ReadOut>());
  if (st) return st;
  CU(cudaMemcpy(en->h_out, en->out.p, sizeof(ReadOut), cudaMemcpyDeviceToHost));
  const ReadOut& r = *en->h_out;
  if (r.status != kOk) return r.status;
  if (r.has_score) {
    if (score) *score = r.score;
    if (score_written) *score_written = 1;
  }
  if (r.n_pairs > pairs_cap) return kCapacity;
  if (r.n_pairs)
    CU(cudaMemcpy(pairs, en->dv.aln_a, (size_t)r.n_pairs * 2 * sizeof(int32_t),
                  cudaMemcpyDeviceToHost));
  *n_pairs = r.n_pairs;
  return kOk;
}

static int32_t add_common(spoa_gb300_graph* g, const int32_t* pairs, uint32_t n_pairs,
                          const char* seq, uint32_t L, const uint32_t* weights,
                          const char* quality) {
  if (L == 0) return kOk;
  int32_t st = graph_reserve(g, L);
  if (st) return st;
  if (g->seq.ensure(L) || g->pairs.ensure((size_t)std::max<uint32_t>(n_pairs, 1) * 8))
    return kNoMemory;
  CU(cudaMemcpy(g->seq.p, seq, L, cudaMemcpyHostToDevice));
  if (n_pairs) CU(cudaMemcpy(g->pairs.p, pairs, (size_t)n_pairs * 8, cudaMemcpyHostToDevice));
  const uint32_t* dw = nullptr;
  const uint8_t* dq = nullptr;
  if (weights || quality) {
    if (g->w.ensure((size_t)L * 4)) return kNoMemory;
    if (weights) {
      CU(cudaMemcpy(g->w.p, weights, (size_t)L * 4, cudaMemcpyHostToDevice));
      dw = g->w.as<uint32_t>();
    } else {
      CU(cudaMemcpy(g->w.p, quality, L, cudaMemcpyHostToDevice));
      dq = g->w.as<uint8_t>();
    }
  }
  k_add<<<1, 32>>>(g->v, g->pairs.as<int32_t>(), n_pairs, g->seq.as<uint8_t>(), L, dw, dq,
                   g->stat.as<int32_t>());
  CU(cudaGetLastError());
  int32_t dst = 0;
  CU(cudaMemcpy(&dst, g->stat.p, 4, cudaMemcpyDeviceToHost));
  st = graph_refresh(g);
  return dst != kOk ? dst : st;
}

int32_t spoa_gb300_graph_add_alignment(spoa_gb300_graph* g, const int32_t* pairs,
                                       uint32_t n_pairs, const char* seq, uint32_t L,
                                       const uint32_t* weights, uint32_t n_weights) {
  if (!g) return kInvalidArgument;
  if (L == 0) return kOk;
  if (weights && n_weights != L) return kUnequalWeights;
  return add_common(g, pairs, n_pairs, seq, L, weights, nullptr);
}

int32_t spoa_gb300_graph_add_alignment_quality(spoa_gb300_graph* g, const int32_t* pairs,
                                               uint32_t n_pairs, const char* seq, uint32_t L,
                                               const char* quality, uint32_t qlen) {
  if (!g) return kInvalidArgument;
  if (L == 0) return kOk;
  if (qlen != L) return kUnequalWeights;
  return add_common(g, pairs, n_pairs, seq, L, nullptr, quality);
}

int32_t spoa_gb300_align_add(spoa_gb300_engine* en, spoa_gb300_graph* g, const char* seq,
                             uint32_t L, const char* quality, int32_t strand, int32_t* score,
                             int32_t* reversed) {
  if (!en || !g) return kInvalidArgument;
  if (L > (uint32_t)INT32_MAX) return kTooLarge;
  if (score) *score = 0;
  if (reversed) *reversed = 0;
  if (L == 0) return kOk;
  const int32_t lanes = g->h.n_nodes ? lanes_for(en->S, L, g->h.n_nodes) : 16;
  if (!lanes) return kOverflow;
  const bool wide = lanes == 8;
  int32_t st = graph_reserve(g, L);
  if (st) return st;
  int cpt, nt;
  st = prepare_read(en, g, L, wide, &cpt, &nt);
  if (st) return st;
  CU(cudaMemcpy(en->seq.p, seq, L, cudaMemcpyHostToDevice));
  const uint8_t* dq = nullptr;
  if (quality) {
    if (en->qual.ensure(L)) return kNoMemory;
    CU(cudaMemcpy(en->qual.p, quality, L, cudaMemcpyHostToDevice));
    dq = en->qual.as<uint8_t>();
  }
  st = SPOA_BY_SUB(en->S.sub, wide, launch_align_add, cpt, nt, en->S, g->v, en->dv,
                   en->seq.as<uint8_t>(), L, dq, strand, en->out.as<ReadOut>(), nullptr,
                   (cudaStream_t)0);
  if (st) return st;
  CU(cudaMemcpy(en->h_out, en->out.p, sizeof(ReadOut), cudaMemcpyDeviceToHost));
  st = graph_refresh(g);
  if (en->h_out->status != kOk) return en->h_out->status;
  if (score) *score = en->h_out->score;
  if (reversed) *reversed = en->h_out->reversed;
  return st;
}

int32_t spoa_gb300_align_add_reads(spoa_gb300_engine* en, spoa_gb300_graph* g, uint32_t n_reads,
                                   const char* seqs, const uint64_t* seq_off, const char* quals,
                                   int32_t strand, int32_t* scores, int32_t* reversed,
                                   uint32_t* n_done) {
  if (!en || !g || !seq_off || (n_reads && !seqs)) return kInvalidArgument;
  if (n_done) *n_done = 0;
  if (!n_reads) return kOk;
  uint64_t sum = 0;
  uint32_t lmax = 1;
  for (uint32_t r = 0; r < n_reads; ++r) {
    if (seq_off[r + 1] < seq_off[r]) return kInvalidArgument;
    const uint64_t L = seq_off[r + 1] - seq_off[r];
    if (L > (uint64_t)INT32_MAX) return kTooLarge;
    lmax = std::max<uint32_t>(lmax, (uint32_t)L);
    sum += L;
  }
  // room for every read, and one width and tile for the whole chain: int32
  // when the reference's rule could pick it for any read (the int32 kernel
  // gives int16-width reads the same results)
  const uint64_t vmax = (uint64_t)g->h.n_nodes + sum;
  const int32_t lanes = lanes_for(en->S, lmax, (uint32_t)std::min<uint64_t>(vmax, 0xFFFFFFFFu));
  const bool wide = lanes != 16;
  int32_t st = graph_reserve(g, sum, n_reads);
  if (st) return st;
  int cpt, nt;
  if (!latency_tile(lmax, wide, &cpt, &nt)) return kTooLarge;
  st = engine_reserve(en, (uint32_t)std::min<uint64_t>(vmax + 1, 0xFFFFFFF0u), (uint32_t)(cpt * nt),
                      (uint32_t)std::min<uint64_t>((uint64_t)g->h.n_edges + sum + n_reads +
                                                       vmax + 2, 0xFFFFFFF0u));
  if (st) return st;
  DeviceBuf d_seqs, d_quals, d_out;
  const uint64_t base = seq_off[0];
  if (d_seqs.ensure(std::max<uint64_t>(sum, 1)) || d_out.ensure(sizeof(ReadOut) * n_reads) ||
      (quals && d_quals.ensure(std::max<uint64_t>(sum, 1))))
    return kNoMemory;
  cudaStream_t s = nullptr;
  CU(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  struct Cleanup {
    cudaStream_t s;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    ~Cleanup() {
      if (exec) cudaGraphExecDestroy(exec);
      if (graph) cudaGraphDestroy(graph);
      cudaStreamDestroy(s);
    }
  } c{s};
  CU(cudaMemcpyAsync(d_seqs.p, seqs + base, sum, cudaMemcpyHostToDevice, s));
  if (quals) CU(cudaMemcpyAsync(d_quals.p, quals + base, sum, cudaMemcpyHostToDevice, s));
  CU(cudaStreamSynchronize(s));
  // the per-read loop, one launch per read in order, recorded into a graph
  ReadOut* out = d_out.as<ReadOut>();
  CU(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  for (uint32_t r = 0; r < n_reads && st == kOk; ++r) {
    const uint64_t o = seq_off[r] - base;
    st = SPOA_BY_SUB(en->S.sub, wide, launch_align_add, cpt, nt, en->S, g->v, en->dv,
                     d_seqs.as<uint8_t>() + o, (uint32_t)(seq_off[r + 1] - seq_off[r]),
                     quals ? d_quals.as<uint8_t>() + o : nullptr, strand, out + r,
                     r ? out + r - 1 : nullptr, s);
  }
  const cudaError_t ec = cudaStreamEndCapture(s, &c.graph);
  if (st) return st;
  CU(ec);
  CU(cudaGraphInstantiate(&c.exec, c.graph, 0));
  CU(cudaGraphLaunch(c.exec, s));
  std::vector<ReadOut> h(n_reads);
  CU(cudaMemcpyAsync(h.data(), out, sizeof(ReadOut) * n_reads, cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  st = graph_refresh(g);
  uint32_t done = 0;
  for (; done < n_reads && h[done].status == kOk; ++done) {
    if (scores) scores[done] = h[done].score;
    if (reversed) reversed[done] = h[done].reversed;
  }
  if (n_done) *n_done = done;
  if (done < n_reads) return h[done].status;
  return st;
}

int32_t spoa_gb300_graph_consensus(spoa_gb300_graph* g, char* out, uint32_t cap,
                                   uint32_t* len) {
  if (!g || !len) return kInvalidArgument;
  DeviceBuf buf, n;
  if (buf.ensure(std::max<uint32_t>(g->h.n_nodes, 1)) || n.ensure(4)) return kNoMemory;
  k_consensus<<<1, 32>>>(g->v, buf.as<uint8_t>(), g->h.n_nodes, n.as<uint32_t>());
  CU(cudaGetLastError());
  CU(cudaMemcpy(len, n.p, 4, cudaMemcpyDeviceToHost));
  if (*len && out) CU(cudaMemcpy(out, buf.p, std::min(*len, cap), cudaMemcpyDeviceToHost));
  return graph_refresh(g);
}

int32_t spoa_gb300_graph_msa(spoa_gb300_graph* g, int32_t include_consensus, char* out,
                             uint64_t cap, uint32_t* rows, uint32_t* cols) {
  if (!g || !rows || !cols) return kInvalidArgument;
  const uint64_t need = (uint64_t)(g->h.n_seqs + 1) * std::max<uint32_t>(g->h.n_nodes, 1);
  DeviceBuf buf, dims, st;
  if (buf.ensure(need) || dims.ensure(8) || st.ensure(4)) return kNoMemory;
  k_msa<<<1, 256>>>(g->v, include_consensus, buf.as<uint8_t>(), need, dims.as<uint32_t>(),
                    st.as<int32_t>());
  CU(cudaGetLastError());
  uint32_t d[2];
  int32_t s = 0;
  CU(cudaMemcpy(d, dims.p, 8, cudaMemcpyDeviceToHost));
  CU(cudaMemcpy(&s, st.p, 4, cudaMemcpyDeviceToHost));
  if (s != kOk) return s;
  *rows = d[0];
  *cols = d[1];
  const uint64_t bytes = (uint64_t)d[0] * d[1];
  if (bytes > cap) return kCapacity;
  if (bytes && out) CU(cudaMemcpy(out, buf.p, bytes, cudaMemcpyDeviceToHost));
  return graph_refresh(g);
}

int32_t spoa_gb300_graph_counts(const spoa_gb300_graph* g, uint32_t* nodes, uint32_t* edges,
                                uint32_t* seqs, uint32_t* consensus, uint32_t* labels,
                                uint32_t* num_codes) {
  if (!g) return kInvalidArgument;
  if (nodes) *nodes = g->h.n_nodes;
  if (edges) *edges = g->h.n_edges;
  if (seqs) *seqs = g->h.n_seqs;
  if (consensus) *consensus = g->h.n_consensus;
  if (labels) *labels = g->h.n_labels;
  if (num_codes) *num_codes = g->h.num_codes;
  return kOk;
}

int32_t spoa_gb300_graph_export(const spoa_gb300_graph* g, uint8_t* chars, uint8_t* codes,
                                uint32_t* in_off, uint32_t* in_edges, uint32_t* out_off,
                                uint32_t* out_edges, uint32_t* al_off, uint32_t* al_nodes,
                                uint32_t* e_tail, uint32_t* e_head, int64_t* e_weight,
                                uint32_t* lab_off, uint32_t* labels, uint32_t* rank,
                                uint32_t* seq_begin, uint32_t* consensus, int32_t* coder,
                                int32_t* decoder) {
  if (!g) return kInvalidArgument;
  const GraphHeader& h = g->h;
  const uint64_t N = h.n_nodes, E = h.n_edges, Lb = h.n_labels, S = h.n_seqs,
                 C = h.n_consensus, A = N * g->caps.aligned;
  struct Item { void* host; uint64_t bytes; };
  Item items[18] = {{chars, N}, {codes, N}, {in_off, 4 * (N + 1)}, {in_edges, 4 * E},
                    {out_off, 4 * (N + 1)}, {out_edges, 4 * E}, {al_off, 4 * (N + 1)},
                    {al_nodes, 4 * A}, {e_tail, 4 * E}, {e_head, 4 * E}, {e_weight, 8 * E},
                    {lab_off, 4 * (E + 1)}, {labels, 4 * Lb}, {rank, 4 * N},
                    {seq_begin, 4 * S}, {consensus, 4 * C}, {coder, 1024}, {decoder, 1024}};
  uint64_t total = 0, offs[18];
  for (int k = 0; k < 18; ++k) {
    offs[k] = total;
    total = align_up(total + std::max<uint64_t>(items[k].bytes, 8), 256);
  }
  DeviceBuf buf;
  if (buf.ensure(total)) return kNoMemory;
  uint8_t* b = buf.as<uint8_t>();
  ExportPtrs x;
  void** slots[18] = {(void**)&x.chars, (void**)&x.codes, (void**)&x.in_off, (void**)&x.in_edges,
                      (void**)&x.out_off, (void**)&x.out_edges, (void**)&x.al_off,
                      (void**)&x.al_nodes, (void**)&x.e_tail, (void**)&x.e_head,
                      (void**)&x.e_weight, (void**)&x.lab_off, (void**)&x.labels, (void**)&x.rank,
                      (void**)&x.seq_begin, (void**)&x.consensus, (void**)&x.coder,
                      (void**)&x.decoder};
  for (int k = 0; k < 18; ++k) *slots[k] = items[k].host ? b + offs[k] : nullptr;
  k_export<<<1, 32>>>(g->v, x);
  CU(cudaGetLastError());
  for (int k = 0; k < 18; ++k)
    if (items[k].host && items[k].bytes)
      CU(cudaMemcpy(items[k].host, b + offs[k], items[k].bytes, cudaMemcpyDeviceToHost));
  return kOk;
}

int32_t spoa_gb300_graph_gfa(const spoa_gb300_graph* g, const char* const* headers,
                             const uint8_t* is_reversed, int32_t include_consensus, char* out,
                             uint64_t cap, uint64_t* len) {
  if (!g || !len) return kInvalidArgument;
  const GraphHeader& h = g->h;
  const uint32_t N = h.n_nodes, E = h.n_edges;
  std::vector<uint8_t> chars(N + 1);
  std::vector<uint32_t> out_off(N + 2), out_e(E + 1), head(E + 1), lab_off(E + 2),
      labels(h.n_labels + 1), sb(h.n_seqs + 1), cons(h.n_consensus + 1);
  std::vector<int64_t> weight(E + 1);
  const int32_t st = spoa_gb300_graph_export(g, chars.data(), nullptr, nullptr, nullptr,
                                             out_off.data(), out_e.data(), nullptr, nullptr,
                                             nullptr, head.data(), weight.data(), lab_off.data(),
                                             labels.data(), nullptr, sb.data(), cons.data(),
                                             nullptr, nullptr);
  if (st) return st;
  GfaGraph gg{N, h.n_seqs, h.n_consensus, chars.data(), out_off.data(), out_e.data(),
              head.data(), weight.data(), lab_off.data(), labels.data(), sb.data(), cons.data()};
  const std::string text = gfa_text(gg, headers, is_reversed, include_consensus != 0);
  *len = text.size();
  if (!out) return kOk;
  if (text.size() > cap) return kCapacity;
  std::memcpy(out, text.data(), text.size());
  return kOk;
}

int32_t spoa_gb300_graph_subgraph(const spoa_gb300_graph* g, uint32_t begin, uint32_t end,
                                  spoa_gb300_graph* out, uint32_t* subgraph_to_graph,
                                  uint32_t map_len) {
  if (!g || !out || out == g || !subgraph_to_graph) return kInvalidArgument;
  const uint32_t nn = g->h.n_nodes;
  if (begin >= nn || end >= nn || map_len < nn) return kInvalidArgument;
  int32_t st = spoa_gb300_graph_clear(out);
  if (st) return st;
  // room for all of g: the subgraph holds at most its nodes and edges
  st = graph_reserve(out, std::max<uint64_t>(nn, g->h.n_edges), 1);
  if (st) return st;
  // each node of the set is expanded once and pushes its in-edge tails and
  // aligned nodes
  const uint64_t stack_cap = (uint64_t)g->h.n_edges + (uint64_t)nn * g->caps.aligned + 1;
  DeviceBuf scratch;
  if (scratch.ensure(4 * (2 * (uint64_t)nn + stack_cap))) return kNoMemory;
  uint32_t* gid = scratch.as<uint32_t>();
  uint32_t* map = gid + nn;
  uint32_t* stack = map + nn;
  k_subgraph<<<1, 256>>>(g->v, out->v, begin, end, gid, stack, stack_cap, map,
                         out->stat.as<int32_t>());
  CU(cudaGetLastError());
  int32_t dst = kOk;
  CU(cudaMemcpy(&dst, out->stat.p, sizeof(dst), cudaMemcpyDeviceToHost));
  if (dst != kOk) {
    spoa_gb300_graph_clear(out);
    return dst;
  }
  st = graph_refresh(out);
  if (st) return st;
  const uint32_t ns = out->h.n_nodes;
  if (ns) CU(cudaMemcpy(subgraph_to_graph, map, 4 * (uint64_t)ns, cudaMemcpyDeviceToHost));
  for (uint32_t k = ns; k < nn; ++k) subgraph_to_graph[k] = 0xFFFFFFFFu;
  return kOk;
}

// ---- graph persistence -----------------------------------------------------
// The fields the reference's Graph::save archives (include/spoa/graph.hpp:
// 188-233), in this library's own little-endian layout:
//   "SPOAGB01"                       magic and version
//   u32 num_codes, i32 coder[256], i32 decoder[256]
//   u32 N, u8 code[N]                nodes in id order
//   u32 E, E x {u32 tail, u32 head, i64 weight, u32 n, u32 label[n]}
//   u32 S, u32 seq_begin[S]
//   u32 P, P x {u32 a, u32 b}        aligned pairs, a < b, in node order
//   u32 R, u32 rank_to_node[R]
//   u32 C, u32 consensus[C]
}  // extern "C"

namespace {

constexpr char kGraphMagic[8] = {'S', 'P', 'O', 'A', 'G', 'B', '0', '1'};

struct Writer {
  uint8_t* out;
  uint64_t cap, n = 0;
  void raw(const void* p, uint64_t bytes) {
    if (out && bytes && n + bytes <= cap) std::memcpy(out + n, p, bytes);
    n += bytes;
  }
  template <typename T> void put(T v) { raw(&v, sizeof(v)); }
};

struct Reader {
  const uint8_t* p;
  uint64_t size, n = 0;
  bool ok = true;
  bool raw(void* dst, uint64_t bytes) {
    if (!ok || bytes > size - n) return ok = false;
    if (!bytes) return true;
    std::memcpy(dst, p + n, bytes);
    n += bytes;
    return true;
  }
  template <typename T> T get() {
    T v{};
    raw(&v, sizeof(v));
    return v;
  }
  // a count of items of `bytes` each that the rest of the buffer can hold
  uint32_t count(uint64_t bytes) {
    const uint32_t c = get<uint32_t>();
    if (ok && (uint64_t)c * bytes > size - n) ok = false;
    return ok ? c : 0;
  }
};

}  // namespace

extern "C" {

int32_t spoa_gb300_graph_save(const spoa_gb300_graph* g, uint8_t* out, uint64_t cap,
                              uint64_t* size) {
  if (!g || !size) return kInvalidArgument;
  const GraphHeader& h = g->h;
  const uint32_t N = h.n_nodes, E = h.n_edges, S = h.n_seqs, C = h.n_consensus;
  std::vector<uint8_t> codes(N + 1);
  std::vector<uint32_t> al_off(N + 1), al((uint64_t)N * g->caps.aligned + 1), tail(E + 1),
      head(E + 1), lab_off(E + 1), labels(h.n_labels + 1), rank(N + 1), sb(S + 1), cons(C + 1);
  std::vector<int64_t> weight(E + 1);
  std::vector<int32_t> coder(256), decoder(256);
  int32_t st = spoa_gb300_graph_export(g, nullptr, codes.data(), nullptr, nullptr, nullptr, nullptr,
                                       al_off.data(), al.data(), tail.data(), head.data(),
                                       weight.data(), lab_off.data(), labels.data(), rank.data(),
                                       sb.data(), cons.data(), coder.data(), decoder.data());
  if (st) return st;
  Writer w{out, out ? cap : 0};
  w.raw(kGraphMagic, sizeof(kGraphMagic));
  w.put<uint32_t>(h.num_codes);
  w.raw(coder.data(), 1024);
  w.raw(decoder.data(), 1024);
  w.put<uint32_t>(N);
  w.raw(codes.data(), N);
  w.put<uint32_t>(E);
  for (uint32_t e = 0; e < E; ++e) {
    w.put<uint32_t>(tail[e]);
    w.put<uint32_t>(head[e]);
    w.put<int64_t>(weight[e]);
    w.put<uint32_t>(lab_off[e + 1] - lab_off[e]);
    w.raw(labels.data() + lab_off[e], 4ull * (lab_off[e + 1] - lab_off[e]));
  }
  w.put<uint32_t>(S);
  w.raw(sb.data(), 4ull * S);
  uint32_t P = 0;
  for (uint32_t v = 0; v < N; ++v)
    for (uint32_t k = al_off[v]; k < al_off[v + 1]; ++k) P += v < al[k];
  w.put<uint32_t>(P);
  for (uint32_t v = 0; v < N; ++v)
    for (uint32_t k = al_off[v]; k < al_off[v + 1]; ++k)
      if (v < al[k]) {
        w.put<uint32_t>(v);
        w.put<uint32_t>(al[k]);
      }
  w.put<uint32_t>(N);
  w.raw(rank.data(), 4ull * N);
  w.put<uint32_t>(C);
  w.raw(cons.data(), 4ull * C);
  *size = w.n;
  return out && w.n > cap ? kCapacity : kOk;
}

int32_t spoa_gb300_graph_load(spoa_gb300_graph* g, const uint8_t* in, uint64_t size) {
  if (!g || (!in && size)) return kInvalidArgument;
  Reader r{in, size};
  char magic[8];
  if (!r.raw(magic, 8) || std::memcmp(magic, kGraphMagic, 8) != 0) return kInvalidArgument;
  const uint32_t num_codes = r.get<uint32_t>();
  std::vector<int32_t> coder(256), decoder(256);
  r.raw(coder.data(), 1024);
  r.raw(decoder.data(), 1024);
  const uint32_t N = r.count(1);
  std::vector<uint8_t> codes(N + 1);
  r.raw(codes.data(), N);
  const uint32_t E = r.count(20);
  std::vector<uint32_t> tail(E + 1), head(E + 1), lab_off(E + 1, 0), labels;
  std::vector<int64_t> weight(E + 1);
  for (uint32_t e = 0; e < E && r.ok; ++e) {
    tail[e] = r.get<uint32_t>();
    head[e] = r.get<uint32_t>();
    weight[e] = r.get<int64_t>();
    const uint32_t nl = r.count(4);
    labels.resize(labels.size() + nl);
    r.raw(labels.data() + labels.size() - nl, 4ull * nl);
    lab_off[e + 1] = (uint32_t)labels.size();
    if (tail[e] >= N || head[e] >= N) r.ok = false;
  }
  const uint32_t S = r.count(4);
  std::vector<uint32_t> sb(S + 1);
  r.raw(sb.data(), 4ull * S);
  const uint32_t P = r.count(8);
  std::vector<uint32_t> pairs(2ull * P + 1);
  r.raw(pairs.data(), 8ull * P);
  const uint32_t R = r.count(4);
  std::vector<uint32_t> rank(R + 1);
  r.raw(rank.data(), 4ull * R);
  const uint32_t C = r.count(4);
  std::vector<uint32_t> cons(C + 1);
  r.raw(cons.data(), 4ull * C);
  if (!r.ok || r.n != size || R != N || C > N || labels.size() >= 0xFFFFFFF0ull)
    return kInvalidArgument;
  // every id in range, ranks a permutation, aligned lists within capacity
  std::vector<uint8_t> seen(N + 1, 0);
  std::vector<uint32_t> deg(N + 1, 0);
  for (uint32_t k = 0; k < R; ++k) {
    if (rank[k] >= N || seen[rank[k]]) return kInvalidArgument;
    seen[rank[k]] = 1;
  }
  for (uint32_t k = 0; k < S; ++k)
    if (sb[k] >= N) return kInvalidArgument;
  for (uint32_t k = 0; k < C; ++k)
    if (cons[k] >= N) return kInvalidArgument;
  for (uint32_t k = 0; k < 2 * P; ++k) {
    if (pairs[k] >= N) return kInvalidArgument;
    if (++deg[pairs[k]] > g->caps.aligned) return kCapacity;
  }
  for (uint32_t k = 0; k < P; ++k)
    if (pairs[2 * k] == pairs[2 * k + 1]) return kInvalidArgument;
  for (int k = 0; k < 256; ++k)
    if (coder[k] < -1 || coder[k] > 255 || decoder[k] < -1 || decoder[k] > 255)
      return kInvalidArgument;
  int32_t st = spoa_gb300_graph_clear(g);
  if (st) return st;
  const uint64_t Lb = labels.size();
  st = graph_reserve(g, std::max<uint64_t>({N, E, Lb}), std::max<uint32_t>(S, 1));
  if (st) return st;
  // one device buffer for every array
  const uint64_t items[] = {N, 4ull * E, 4ull * E, 8ull * E, 4ull * (E + 1), 4 * Lb, 4ull * S,
                            8ull * P, 4ull * N, 4ull * C, 1024, 1024};
  const void* src[] = {codes.data(), tail.data(), head.data(), weight.data(), lab_off.data(),
                       labels.data(), sb.data(), pairs.data(), rank.data(), cons.data(),
                       coder.data(), decoder.data()};
  uint64_t offs[12], total = 0;
  for (int k = 0; k < 12; ++k) {
    offs[k] = total;
    total = align_up(total + std::max<uint64_t>(items[k], 8), 256);
  }
  DeviceBuf buf;
  if (buf.ensure(total)) return kNoMemory;
  uint8_t* b = buf.as<uint8_t>();
  for (int k = 0; k < 12; ++k)
    if (items[k]) CU(cudaMemcpy(b + offs[k], src[k], items[k], cudaMemcpyHostToDevice));
  ImportArgs a;
  a.n_nodes = N;
  a.n_edges = E;
  a.n_seqs = S;
  a.n_pairs = P;
  a.n_consensus = C;
  a.num_codes = num_codes;
  a.codes = b + offs[0];
  a.e_tail = reinterpret_cast<const uint32_t*>(b + offs[1]);
  a.e_head = reinterpret_cast<const uint32_t*>(b + offs[2]);
  a.e_weight = reinterpret_cast<const int64_t*>(b + offs[3]);
  a.lab_off = reinterpret_cast<const uint32_t*>(b + offs[4]);
  a.labels = reinterpret_cast<const uint32_t*>(b + offs[5]);
  a.seq_begin = reinterpret_cast<const uint32_t*>(b + offs[6]);
  a.pairs = reinterpret_cast<const uint32_t*>(b + offs[7]);
  a.rank = reinterpret_cast<const uint32_t*>(b + offs[8]);
  a.consensus = reinterpret_cast<const uint32_t*>(b + offs[9]);
  a.coder = reinterpret_cast<const int32_t*>(b + offs[10]);
  a.decoder = reinterpret_cast<const int32_t*>(b + offs[11]);
  k_import<<<1, 32>>>(g->v, a, g->stat.as<int32_t>());
  CU(cudaGetLastError());
  int32_t dst = kOk;
  CU(cudaMemcpy(&dst, g->stat.p, sizeof(dst), cudaMemcpyDeviceToHost));
  if (dst != kOk) {
    spoa_gb300_graph_clear(g);
    return dst;
  }
  return graph_refresh(g);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// batched windows
// ---------------------------------------------------------------------------
namespace {



// One persistent launch over a group of windows that share a tile (columns
// per thread x threads) and a lane width.
struct Pass {
  bool wide = false;              // int32 kernel
  std::vector<uint32_t> windows;  // window ids in queue order
  GraphCaps gcaps{};
  DpCaps dcaps{};
  int cpt = 0, nt = 0, ctas = 0;
  int segs = 1;             // strips per thread (dp_forward_seg when > 1)
  int wpc = 1;              // windows per CTA (batch_cta_mw when > 1)
  uint64_t stride = 0;
  int tuned_cpt = 0, tuned_nt = 0;  // tile chosen by the tuner (0: the default)
  int tuned_wpc = 0, tuned_regs = 0;  // windows per CTA and register cap chosen by the tuner
  int regs = 0;             // 128: the one-warp 16-bit kernel with 128 registers
  int cl = 1;               // CTAs per window (k_batch_cl when > 1); ctas counts clusters
  int cls = 0;              // length class
  double work = 0;          // estimated DP work (sum of read lengths x longest read)
  uint64_t arena_off = 0;   // byte offset of this pass's arenas in the batch arena
  uint32_t work_off = 0;    // offset of its window list in the device work array
};

// How one window runs next: lane width and graph-node capacity of its arena
// (a window that outgrows it is rerun with twice the nodes, up to the sum of
// its read lengths, which no graph exceeds).
struct WindowPlan {
  bool wide = false;
  bool many_aligned = false;  // room for 63 aligned nodes per node, not 4
  uint64_t nodes = 0;
};

template <typename T>
int32_t upload(DeviceBuf& d, const T* h, size_t count, cudaStream_t s) {
  if (d.ensure(std::max<size_t>(count * sizeof(T), 8))) return kNoMemory;
  if (count && h) CU(cudaMemcpyAsync(d.p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
  return kOk;
}

}  // namespace

struct spoa_gb300_batch {
  spoa_gb300_batch_desc desc{};
  Scoring base{};
  uint32_t n_windows = 0, n_reads = 0;
  std::vector<uint32_t> wro;
  std::vector<uint64_t> seq_off;
  std::vector<uint32_t> lmax, nreads;
  std::vector<uint64_t> sumlen;
  DeviceBuf d_seqs, d_seq_off, d_quals, d_wro, d_wtype, d_wstrand;
  DeviceBuf d_work, d_queue, d_scores, d_rev, d_cons, d_cons_off, d_cons_len, d_status;
  DeviceBuf d_aln, d_aln_off, d_aln_len, d_msa, d_msa_off, d_msa_rows, d_msa_cols, d_cells;
  DeviceBuf arena;
  std::vector<uint64_t> aln_off, msa_off;
  std::vector<uint64_t> cons_off;  // first-pass regions
  // host results
  std::vector<int32_t> h_scores, h_status, h_aln;
  std::vector<uint8_t> h_rev;
  std::vector<char> h_cons, h_msa;
  std::vector<uint64_t> h_cons_off, h_aln_off;
  std::vector<uint32_t> h_msa_rows, h_msa_cols, h_aln_len;
  std::vector<Pass> passes;           // first launch: one pass per tile bucket
  uint64_t budget = 0;                // device bytes for arenas
  std::vector<cudaStream_t> streams;  // one per concurrent pass
  ~spoa_gb300_batch() {
    for (cudaStream_t st : streams) cudaStreamDestroy(st);
  }
  std::vector<WindowPlan> plan0;      // per window, as created
  std::vector<std::string> retry_cons;  // consensus of windows that ran again
  std::vector<uint8_t> retried;         // per window: retry_cons holds its consensus
  float kernel_ms = 0;
  int launches = 0;
  uint64_t cells = 0;
  int sm_count = 0;
  int device = 0;
};

namespace {

// Capacities of one window's arenas (graph + DP) for a tile: graph nodes
// (at most the sum of the read lengths, which no graph exceeds), edges,
// labels, sequences and aligned-node slots; returns the bytes per CTA.
uint64_t arena_caps(int32_t sub, bool wide, int cpt, int nt, uint64_t nodes, uint64_t maxsum,
                    uint32_t maxreads, bool many_aligned, GraphCaps* gc, DpCaps* dc) {
  nodes = std::min<uint64_t>(nodes, maxsum + 1);
  gc->nodes = (uint32_t)nodes;
  gc->edges = (uint32_t)std::min<uint64_t>(maxsum + 2, 4 * nodes + 64);
  gc->labels = (uint32_t)(maxsum + 2);
  gc->seqs = maxreads + 1;
  gc->aligned = many_aligned ? 63 : 4;  // DNA columns hold at most 5 codes; more reruns
  *dc = DpCaps{(uint32_t)nodes + 1, (uint32_t)(cpt * nt), gc->edges + (uint32_t)nodes + 2, sub,
               wide ? 4 : 2};
  GraphView gv;
  DpView dv;
  return align_up(graph_layout(nullptr, *gc, &gv), 256) + align_up(dp_layout(nullptr, *dc, &dv), 256);
}

int32_t plan_pass(spoa_gb300_batch* b, Pass* p, const std::vector<WindowPlan>& wp) {
  const spoa_gb300_batch_desc& d = b->desc;
  uint32_t L = 1, maxreads = 1;
  uint64_t maxsum = 1, wnodes = 1;
  bool many_aligned = false;
  for (uint32_t w : p->windows) {
    L = std::max(L, b->lmax[w]);
    maxsum = std::max(maxsum, b->sumlen[w]);
    maxreads = std::max(maxreads, b->nreads[w]);
    wnodes = std::max(wnodes, wp[w].nodes);
    many_aligned = many_aligned || wp[w].many_aligned;
  }
  int cpt = d.columns_per_thread, nt = d.threads_per_window, segs = 1, cl = 1;
  const bool forced = cpt > 0 && nt > 0;
  if (p->wide && !forced && d.cluster != 1 &&
      cluster_tile(L, p->windows.size(), b->sm_count, d.cluster, &cl, &nt)) {
    cpt = kClCpt;  // a thread-block cluster per window
  } else if (p->tuned_cpt > 0 && (uint64_t)p->tuned_cpt * p->tuned_nt >= L) {
    cpt = p->tuned_cpt;
    nt = p->tuned_nt;
  }
  if (cpt <= 0 || nt <= 0 || (p->wide && !cpt_supported<int32_t>(cpt)) ||
      (!p->wide && !cpt_supported<int16_t>(cpt))) {
    // default tile; 32-bit rows past one 12-column strip per thread go to
    // the segmented kernel
    if (p->wide && L > (uint32_t)kSegCpt * 512) {
      if (!seg_tile(L, &cpt, &nt, &segs)) return kTooLarge;
    } else if (!throughput_tile(L, p->wide, &cpt, &nt)) {
      return kTooLarge;
    }
  } else if ((uint64_t)cpt * nt * cl < L) {
    return kTooLarge;
  }
  uint64_t nodes = d.max_nodes ? std::max<uint64_t>(d.max_nodes, wnodes) : wnodes;
  GraphCaps gc;
  DpCaps dc;
  uint64_t stride =
      arena_caps(b->base.sub, p->wide, cpt * segs * cl, nt, nodes, maxsum, maxreads, many_aligned,
                 &gc, &dc);
  // several windows per CTA: 16-bit lanes, single-strip tiles (the tuner's
  // choice for the class, else the descriptor's)
  const int want_wpc = p->tuned_wpc > 0 ? p->tuned_wpc : d.windows_per_cta;
  const int wpc = (want_wpc == 2 || want_wpc == 4) && !p->wide && segs == 1 && cl == 1 ? want_wpc : 1;
  if (wpc > 1) {
    DpView dv;
    stride = align_up(mw_layout(nullptr, wpc, gc, dc, &dv, nullptr, nullptr, nullptr), 256);
  }
  // 128 registers: one-warp 16-bit single-window tiles, when the tuner chose it
  const int regs = p->tuned_regs == 128 && !p->wide && segs == 1 && wpc == 1 && nt == 32 ? 128 : 0;
  int blocks = 1;
  if (cl > 1) {
    // clusters resident on the whole device, not per SM
    int clusters = 1;
    if (SPOA_BY_SUB16(b->base.sub, occupancy_batch_cl, cl, nt, &clusters)) return kCuda;
    uint64_t n = std::max(clusters, 1);
    n = std::min<uint64_t>(n, std::max<uint64_t>(1, b->budget / stride));
    n = std::min<uint64_t>(n, p->windows.size());
    p->gcaps = gc;
    p->dcaps = dc;
    p->cpt = cpt;
    p->nt = nt;
    p->segs = 1;
    p->wpc = 1;
    p->regs = 0;
    p->cl = cl;
    p->ctas = (int)std::max<uint64_t>(n, 1);
    p->stride = stride;
    return kOk;
  }
  if (segs > 1 ? SPOA_BY_SUB32(b->base.sub, occupancy_batch_seg, segs, nt, &blocks)
      : wpc > 1 ? SPOA_BY_SUB16(b->base.sub, occupancy_batch_mw, cpt, nt, wpc, &blocks)
      : regs ? SPOA_BY_SUB16(b->base.sub, occupancy_batch_r128, cpt, &blocks)
                : SPOA_BY_SUB(b->base.sub, p->wide, occupancy_batch, cpt, nt, &blocks))
    return kCuda;
  blocks = std::max(blocks, 1);
  uint64_t by_mem = std::max<uint64_t>(1, b->budget / stride);
  uint64_t ctas = d.ctas > 0 ? (uint64_t)d.ctas : (uint64_t)b->sm_count * blocks;
  ctas = std::min<uint64_t>(ctas, by_mem);
  ctas = std::min<uint64_t>(ctas, (p->windows.size() + wpc - 1) / wpc);
  p->gcaps = gc;
  p->dcaps = dc;
  p->cpt = cpt;
  p->nt = nt;
  p->segs = segs;
  p->wpc = wpc;
  p->regs = regs;
  p->cl = 1;
  p->ctas = (int)std::max<uint64_t>(ctas, 1);
  p->stride = stride;
  return kOk;
}

BatchArgs make_args(spoa_gb300_batch* b, const Pass& p, uint8_t* cons, const uint64_t* cons_off) {
  BatchArgs a{};
  a.base = b->base;
  a.win_type = b->desc.window_type ? b->d_wtype.as<int8_t>() : nullptr;
  a.win_strand = b->desc.window_strand ? b->d_wstrand.as<int8_t>() : nullptr;
  a.n_windows = b->n_windows;
  a.win_read_off = b->d_wro.as<uint32_t>();
  a.seqs = b->d_seqs.as<uint8_t>();
  a.seq_off = b->d_seq_off.as<uint64_t>();
  a.quals = b->desc.quals ? b->d_quals.as<uint8_t>() : nullptr;
  a.work = b->d_work.as<uint32_t>() + p.work_off;
  a.n_work = (uint32_t)p.windows.size();
  a.queue = b->d_queue.as<uint32_t>() + p.work_off;
  a.arena = b->arena.as<uint8_t>() + p.arena_off;
  a.arena_stride = p.stride;
  a.gcaps = p.gcaps;
  a.dcaps = p.dcaps;
  a.read_scores = b->d_scores.as<int32_t>();
  a.read_rev = b->d_rev.as<uint8_t>();
  a.cons = cons;
  a.cons_off = cons_off;
  a.cons_len = b->d_cons_len.as<uint32_t>();
  a.win_status = b->d_status.as<int32_t>();
  if (b->desc.want_alignments) {
    a.aln_out = b->d_aln.as<int32_t>();
    a.aln_off = b->d_aln_off.as<uint64_t>();
    a.aln_len = b->d_aln_len.as<uint32_t>();
  }
  if (b->desc.want_msa) {
    a.msa_out = b->d_msa.as<uint8_t>();
    a.msa_off = b->d_msa_off.as<uint64_t>();
    a.msa_rows = b->d_msa_rows.as<uint32_t>();
    a.msa_cols = b->d_msa_cols.as<uint32_t>();
  }
  a.cells = b->d_cells.as<unsigned long long>();
  a.pred_cells = a.cells + 1;
  return a;
}

int32_t launch_pass(spoa_gb300_batch* b, const Pass& p, int ctas, const BatchArgs& a,
                    cudaStream_t s) {
  ++b->launches;
  if (p.cl > 1) return SPOA_BY_SUB16(b->base.sub, launch_batch_cl, p.cl, p.nt, ctas, a, s);
  if (p.segs > 1) return SPOA_BY_SUB32(b->base.sub, launch_batch_seg, p.segs, p.nt, ctas, a, s);
  if (p.wpc > 1)
    return SPOA_BY_SUB16(b->base.sub, launch_batch_mw, p.cpt, p.nt, p.wpc, ctas, a, s);
  if (p.regs == 128) return SPOA_BY_SUB16(b->base.sub, launch_batch_r128, p.cpt, ctas, a, s);
  return SPOA_BY_SUB(b->base.sub, p.wide, launch_batch, p.cpt, p.nt, ctas, a, s);
}

int32_t run_pass(spoa_gb300_batch* b, const Pass& p, cudaStream_t s, bool plain, uint8_t* cons,
                 const uint64_t* cons_off) {
  if (p.windows.empty()) return kOk;
  CU(cudaMemcpyAsync(b->d_work.as<uint32_t>() + p.work_off, p.windows.data(),
                     p.windows.size() * 4, cudaMemcpyHostToDevice, s));
  CU(cudaMemsetAsync(b->d_queue.as<uint32_t>() + p.work_off, 0, 4 * p.windows.size(), s));
  BatchArgs a = make_args(b, p, cons, cons_off);
  if (!plain) return launch_pass(b, p, p.ctas, a, s);
  for (size_t k = 0; k < p.windows.size(); ++k) {
    BatchArgs one = a;
    one.work = a.work + k;
    one.n_work = 1;
    one.queue = a.queue + k;
    int32_t st = launch_pass(b, p, 1, one, s);
    if (st) return st;
  }
  return kOk;
}

// ---- tile tuner ------------------------------------------------------------
// A tuner choice for one length class: columns per thread x threads, and for
// 16-bit single-strip tiles windows per CTA (batch_cta_mw) and the register
// cap of the one-warp kernel (0: the default).
struct TileChoice {
  int cpt = 0, nt = 0, wpc = 1, regs = 0;
};

// Candidate tiles for windows up to L columns: every columns-per-thread of
// the width with its thread count (a multiple of 32, at most 512), kept when
// its padded row is at most 1.5x the tightest; at most four, tightest first.
std::vector<std::pair<int, int>> tile_candidates(uint32_t L, bool wide) {
  std::vector<std::tuple<uint64_t, int, int>> c;
  const int* cs = wide ? kCpts32 : kCpts16;
  const int nc = wide ? 5 : 6;
  for (int k = 0; k < nc; ++k) {
    const uint64_t t = std::max<uint64_t>(32, ((uint64_t)(L + cs[k] - 1) / cs[k] + 31) / 32 * 32);
    if (t <= 512) c.emplace_back(t * cs[k], cs[k], (int)t);
  }
  std::sort(c.begin(), c.end());
  std::vector<std::pair<int, int>> out;
  for (const auto& x : c)
    if (std::get<0>(x) * 2 <= std::get<0>(c.front()) * 3 && out.size() < 4)
      out.emplace_back(std::get<1>(x), std::get<2>(x));
  return out;
}

// Tiles chosen by timing, per (gap model, width, length class), for the
// life of the process; when SPOA_GB300_TILE_CACHE names a file they are also
// kept there (one "device sub wide class cpt nt" line each) and reused by
// later processes on the same device model.
std::mutex g_tune_mu;
std::map<std::tuple<int, bool, int>, TileChoice> g_tuned;
bool g_tune_loaded = false;

std::string device_tag() {
  int dev = 0;
  cudaDeviceProp prop;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
    cudaGetLastError();
    return "unknown";
  }
  std::string t = prop.name;
  for (char& ch : t)
    if (ch == ' ') ch = '_';
  return t + "_sm" + std::to_string(prop.multiProcessorCount);
}

void load_tile_cache() {  // under g_tune_mu
  if (g_tune_loaded) return;
  g_tune_loaded = true;
  const char* path = std::getenv("SPOA_GB300_TILE_CACHE");
  if (!path) return;
  FILE* f = std::fopen(path, "r");
  if (!f) return;
  const std::string tag = device_tag();
  char line[512], dev[256];
  while (std::fgets(line, sizeof line, f)) {
    int sub, wide, cls;
    TileChoice t;
    const int got = std::sscanf(line, "%255s %d %d %d %d %d %d %d", dev, &sub, &wide, &cls,
                                &t.cpt, &t.nt, &t.wpc, &t.regs);
    if (got < 6) continue;
    if (got < 8) t.wpc = 1, t.regs = 0;  // lines of the tile-only format
    if (tag == dev && t.cpt > 0 && t.nt > 0) g_tuned[std::make_tuple(sub, wide != 0, cls)] = t;
  }
  std::fclose(f);
}

void save_tile(int sub, bool wide, int cls, const TileChoice& t) {  // under g_tune_mu
  g_tuned[std::make_tuple(sub, wide, cls)] = t;
  const char* path = std::getenv("SPOA_GB300_TILE_CACHE");
  if (!path) return;
  if (FILE* f = std::fopen(path, "a")) {
    std::fprintf(f, "%s %d %d %d %d %d %d %d\n", device_tag().c_str(), sub, wide ? 1 : 0, cls,
                 t.cpt, t.nt, t.wpc, t.regs);
    std::fclose(f);
  }
}

bool tuned_tile(int sub, bool wide, int cls, TileChoice* t) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  load_tile_cache();
  auto it = g_tuned.find(std::make_tuple(sub, wide, cls));
  if (it == g_tuned.end()) return false;
  *t = it->second;
  return true;
}

// Groups windows into passes by lane width and length class (longest read
// up to 640 columns, i.e. one warp, then doublings: 1280, 2560, ...); each
// pass takes the tile of its longest read.  Classes are coarse on purpose:
// a persistent pass ends with a tail of its last windows, so fewer, fuller
// passes beat a tighter tile per window.  Passes with the longest windows
// come first.
int32_t make_passes(spoa_gb300_batch* b, const std::vector<uint32_t>& windows,
                    const std::vector<WindowPlan>& wp, std::vector<Pass>* out) {
  const spoa_gb300_batch_desc& d = b->desc;
  std::map<std::tuple<bool, int, int>, std::vector<uint32_t>> groups;
  const bool forced = d.columns_per_thread > 0 && d.threads_per_window > 0;
  for (uint32_t w : windows) {
    const bool wide = wp[w].wide;
    int cls = 0;
    if (!forced)
      for (uint64_t cap = 640; cap < b->lmax[w]; cap *= 2) ++cls;
    groups[std::make_tuple(wide, cls, 0)].push_back(w);
  }
  auto work = [&](uint32_t w) { return (double)b->sumlen[w] * b->lmax[w]; };
  std::vector<std::pair<double, Pass>> ps;
  for (auto& g : groups) {
    Pass p;
    p.wide = std::get<0>(g.first);
    p.cls = std::get<1>(g.first);
    p.windows = std::move(g.second);
    TileChoice tc;
    if (!forced && tuned_tile(b->base.sub, p.wide, p.cls, &tc)) {
      p.tuned_cpt = tc.cpt;
      p.tuned_nt = tc.nt;
      p.tuned_wpc = tc.wpc;
      p.tuned_regs = tc.regs;
    }
    std::stable_sort(p.windows.begin(), p.windows.end(),
                     [&](uint32_t x, uint32_t y) { return work(x) > work(y); });
    double total = 0;
    for (uint32_t w : p.windows) total += work(w);
    p.work = total;
    int32_t st = plan_pass(b, &p, wp);
    if (st) return st;
    ps.emplace_back(total, std::move(p));
  }
  std::stable_sort(ps.begin(), ps.end(),
                   [](const std::pair<double, Pass>& x, const std::pair<double, Pass>& y) {
                     return x.second.dcaps.ld > y.second.dcaps.ld;
                   });
  out->clear();
  for (auto& x : ps) out->push_back(std::move(x.second));
  // The passes of one launch are issued together, each on its own stream,
  // longest windows first: the block scheduler places their CTAs first and
  // the passes of shorter windows fill the rest of the GPU and take over the
  // slots of any pass whose queue runs dry.  Each pass keeps its full CTA
  // count; the arena budget is split in proportion to the passes' work.
  double all = 0;
  for (const Pass& p : *out) all += p.work;
  uint64_t arena = 0, woff = 0;
  for (Pass& p : *out) {
    const double share = all > 0 ? p.work / all : 1.0;
    uint64_t by_mem = std::max<uint64_t>(1, (uint64_t)(share * (double)b->budget) / p.stride);
    if (out->size() > 1)
      p.ctas = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)p.ctas, by_mem));
    p.arena_off = arena;
    arena += align_up(p.stride * (uint64_t)p.ctas, 256);
    p.work_off = (uint32_t)woff;
    woff += p.windows.size();
  }
  if (b->arena.ensure(std::max<uint64_t>(arena, 256))) return kNoMemory;
  return kOk;
}

// Times the candidate tiles of every pass whose class has no tuned tile
// yet, each on the same sample of the pass's windows (its longest, enough to
// fill the GPU), keeps the fastest per window, then re-plans the passes.
// The sample's results are overwritten by the real launch.
int32_t autotune(spoa_gb300_batch* b, cudaStream_t s) {
  bool changed = false;
  cudaEvent_t e0, e1;
  CU(cudaEventCreate(&e0));
  CU(cudaEventCreate(&e1));
  for (const Pass& p : b->passes) {
    TileChoice known;
    if (p.segs > 1 || p.cl > 1 || tuned_tile(b->base.sub, p.wide, p.cls, &known)) continue;
    uint32_t L = 1;
    for (uint32_t w : p.windows) L = std::max(L, b->lmax[w]);
    std::vector<TileChoice> cands;
    for (const auto& c : tile_candidates(L, p.wide)) {
      TileChoice t;
      t.cpt = c.first;
      t.nt = c.second;
      cands.push_back(t);
    }
    // The default tile (fewest padded columns, then fewest threads) comes
    // first; for 16-bit one-warp defaults also two windows per CTA and the
    // 128-register build of the one-warp kernel.
    int dc = 0, dn = 0;
    if (!throughput_tile(L, p.wide, &dc, &dn)) dc = dn = 0;
    std::stable_partition(cands.begin(), cands.end(),
                          [&](const TileChoice& t) { return t.cpt == dc && t.nt == dn; });
    if (!cands.empty() && !p.wide && cands.front().cpt == dc && dn == 32) {
      TileChoice t = cands.front();
      t.wpc = 2;
      cands.push_back(t);
      t.wpc = 1;
      t.regs = 128;
      cands.push_back(t);
    }
    TileChoice best = cands.empty() ? TileChoice{} : cands.front();
    if (cands.size() > 1) {
      // one sample for every candidate: at least four windows per CTA of the
      // candidate with the most CTAs, so the pass's tail does not decide
      Pass q;
      q.wide = p.wide;
      q.cls = p.cls;
      q.windows = p.windows;
      auto take = [&](const TileChoice& t) {
        q.tuned_cpt = t.cpt;
        q.tuned_nt = t.nt;
        q.tuned_wpc = t.wpc;
        q.tuned_regs = t.regs;
        return plan_pass(b, &q, b->plan0);
      };
      size_t n = 1;
      for (const auto& c : cands) {
        int32_t st = take(c);
        if (st) return st;
        n = std::max<size_t>(n, 4 * (size_t)q.ctas * (size_t)q.wpc);
      }
      // evenly spaced over the pass (longest first), so the sample keeps
      // its mix of window sizes
      std::vector<uint32_t> sample;
      const size_t step = std::max<size_t>(1, p.windows.size() / std::max<size_t>(n, 1));
      for (size_t k = 0; k < p.windows.size() && sample.size() < n; k += step)
        sample.push_back(p.windows[k]);
      q.windows = sample;
      // The default (index 0) stays unless another candidate is faster in
      // every one of three rounds by more than 3 %: a single timing can be
      // off (the first launch of a kernel loads its module, clocks still
      // rising, another process), and a choice kept by mistake costs every
      // later launch.
      constexpr int kRounds = 3;
      std::vector<std::vector<float>> ms_of(cands.size());
      for (int round = 0; round < kRounds; ++round) {
        for (size_t k = 0; k < cands.size(); ++k) {
          int32_t st = take(cands[k]);
          if (st) return st;
          if (b->arena.ensure(q.stride * (uint64_t)q.ctas)) return kNoMemory;
          CU(cudaEventRecord(e0, s));
          st = run_pass(b, q, s, false, b->d_cons.as<uint8_t>(), b->d_cons_off.as<uint64_t>());
          if (st) return st;
          CU(cudaEventRecord(e1, s));
          CU(cudaEventSynchronize(e1));
          float ms = 0;
          CU(cudaEventElapsedTime(&ms, e0, e1));
          ms_of[k].push_back(ms);
        }
      }
      const float dmin = *std::min_element(ms_of[0].begin(), ms_of[0].end());
      size_t bi = 0;
      float bmax = dmin;
      for (size_t k = 1; k < cands.size(); ++k) {
        const float kmax = *std::max_element(ms_of[k].begin(), ms_of[k].end());
        if (kmax < 0.97f * dmin && kmax < bmax) {
          bi = k;
          bmax = kmax;
        }
      }
      if (std::getenv("SPOA_GB300_TUNE_LOG")) {
        for (size_t k = 0; k < cands.size(); ++k) {
          std::fprintf(stderr, "tile tuner: sub %d wide %d class %d tile %dx%d wpc %d regs %d ms",
                       (int)b->base.sub, p.wide ? 1 : 0, p.cls, cands[k].cpt, cands[k].nt,
                       cands[k].wpc, cands[k].regs);
          for (float x : ms_of[k]) std::fprintf(stderr, " %.2f", x);
          std::fprintf(stderr, "%s\n", k == bi ? " (kept)" : "");
        }
      }
      best = cands[bi];
    }
    std::lock_guard<std::mutex> lk(g_tune_mu);
    save_tile((int)b->base.sub, p.wide, p.cls, best);
    changed = true;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (changed) {
    std::vector<uint32_t> all(b->n_windows);
    for (uint32_t w = 0; w < b->n_windows; ++w) all[w] = w;
    return make_passes(b, all, b->plan0, &b->passes);
  }
  return kOk;
}

int32_t launch_all(spoa_gb300_batch* b, void* stream, bool plain) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const bool forced = b->desc.columns_per_thread > 0 && b->desc.threads_per_window > 0;
  if (b->desc.autotune && !forced && !plain) {
    int32_t st = autotune(b, s);
    if (st) return st;
  }
  b->launches = 0;
  b->kernel_ms = 0;
  b->retry_cons.clear();
  b->retried.assign(b->n_windows, 0);
  cudaEvent_t e0, e1;
  CU(cudaEventCreate(&e0));
  CU(cudaEventCreate(&e1));
  CU(cudaMemsetAsync(b->d_cells.p, 0, 16, s));
  std::vector<WindowPlan> wp = b->plan0;
  std::vector<Pass> passes = b->passes;
  std::vector<int32_t> status(b->n_windows);
  // consensus regions of rerun windows: the exact bound, in a second buffer
  std::vector<uint64_t> off2(b->n_windows + 1, 0);
  for (uint32_t w = 0; w < b->n_windows; ++w) off2[w + 1] = off2[w] + b->sumlen[w] + 1;
  DeviceBuf cons2, doff2;
  bool rerun = false;
  for (int round = 0; !passes.empty(); ++round) {
    if (round == 1) {
      if (cons2.ensure(off2[b->n_windows] + 8)) return kNoMemory;
      if (upload(doff2, off2.data(), off2.size(), s)) return kNoMemory;
    }
    uint8_t* cons = round == 0 ? b->d_cons.as<uint8_t>() : cons2.as<uint8_t>();
    const uint64_t* coff = round == 0 ? b->d_cons_off.as<uint64_t>() : doff2.as<uint64_t>();
    CU(cudaEventRecord(e0, s));
    if (plain || passes.size() == 1) {
      for (const Pass& p : passes) {
        int32_t st = run_pass(b, p, s, plain, cons, coff);
        if (st) return st;
      }
    } else {
      // fork: every pass on its own stream, joined back into s
      while (b->streams.size() < passes.size()) {
        cudaStream_t st = nullptr;
        CU(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        b->streams.push_back(st);
      }
      cudaEvent_t fork;
      CU(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
      CU(cudaEventRecord(fork, s));
      std::vector<cudaEvent_t> joins(passes.size());
      for (size_t k = 0; k < passes.size(); ++k) {
        CU(cudaStreamWaitEvent(b->streams[k], fork, 0));
        int32_t st = run_pass(b, passes[k], b->streams[k], plain, cons, coff);
        if (st) return st;
        CU(cudaEventCreateWithFlags(&joins[k], cudaEventDisableTiming));
        CU(cudaEventRecord(joins[k], b->streams[k]));
        CU(cudaStreamWaitEvent(s, joins[k], 0));
      }
      cudaEventDestroy(fork);
      for (cudaEvent_t ev : joins) cudaEventDestroy(ev);
    }
    CU(cudaEventRecord(e1, s));
    CU(cudaMemcpyAsync(status.data(), b->d_status.p, 4ull * b->n_windows, cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    float ms = 0;
    CU(cudaEventElapsedTime(&ms, e0, e1));
    b->kernel_ms += ms;
    if (round > 0) {
      // keep the consensus of the windows this round ran
      std::vector<uint32_t> lens(b->n_windows);
      CU(cudaMemcpy(lens.data(), b->d_cons_len.p, 4ull * b->n_windows, cudaMemcpyDeviceToHost));
      std::vector<char> tmp(off2[b->n_windows] + 8);
      CU(cudaMemcpy(tmp.data(), cons2.p, off2[b->n_windows], cudaMemcpyDeviceToHost));
      b->retry_cons.resize(b->n_windows);
      for (const Pass& p : passes)
        for (uint32_t w : p.windows) {
          b->retry_cons[w].assign(tmp.data() + off2[w],
                                  std::min<uint64_t>(lens[w], off2[w + 1] - off2[w]));
          b->retried[w] = 1;
        }
    }
    // windows that need the int32 width or outgrew their arena run again
    std::vector<uint32_t> again;
    for (const Pass& p : passes) {
      for (uint32_t w : p.windows) {
        if (status[w] == kNeedWide) {
          wp[w].wide = true;
          again.push_back(w);
        } else if (status[w] == kCapacity && wp[w].nodes < b->sumlen[w] + 1) {
          wp[w].nodes = std::min<uint64_t>(2 * wp[w].nodes, b->sumlen[w] + 1);
          wp[w].many_aligned = true;
          again.push_back(w);
        } else if (status[w] == kCapacity && !wp[w].many_aligned) {
          wp[w].many_aligned = true;
          again.push_back(w);
        }
      }
    }
    if (!again.empty()) rerun = true;
    int32_t st = make_passes(b, again, wp, &passes);
    if (st) return st;
    if (round > 64) break;  // unreachable: every rerun doubles a bounded capacity
  }
  if (!rerun) b->retry_cons.clear();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return kOk;
}

}  // namespace

extern "C" {

int32_t spoa_gb300_batch_create(const spoa_gb300_batch_desc* d, spoa_gb300_batch** out) {
  if (!d || !out || !d->window_read_off || !d->seq_off || (!d->seqs && d->n_windows))
    return kInvalidArgument;
  *out = nullptr;
  // what the descriptor alone decides is checked before any CUDA call:
  // types, penalties (AlignmentEngine::Create), the window offsets
  if (d->type != kSW && d->type != kNW && d->type != kOV) return kInvalidArgument;
  if (d->g > 0 || d->q > 0 || d->e > 0 || d->c > 0) return kInvalidArgument;
  if (d->window_read_off[0] != 0) return kInvalidArgument;
  for (uint32_t w = 0; w < d->n_windows; ++w) {
    if (d->window_read_off[w + 1] < d->window_read_off[w]) return kInvalidArgument;
    if (d->window_type) {
      const int8_t t = d->window_type[w];
      if (t != kSW && t != kNW && t != kOV) return kInvalidArgument;
    }
  }
  const int dev = resolve_device(d->device_set, d->device);
  if (dev < 0) return d->device_set ? kInvalidArgument : kCuda;
  DeviceGuard guard(dev);
  if (!guard.ok) return kCuda;
  spoa_gb300_engine* en = nullptr;
  int32_t st = spoa_gb300_engine_create(d->type, d->m, d->n, d->g, d->e, d->q, d->c, &en);
  if (st) return st;
  Scoring base = en->S;
  spoa_gb300_engine_destroy(en);
  auto* b = new (std::nothrow) spoa_gb300_batch();
  if (!b) return kNoMemory;
  b->desc = *d;
  b->device = dev;
  b->base = base;
  b->n_windows = d->n_windows;
  b->wro.assign(d->window_read_off, d->window_read_off + d->n_windows + 1);
  b->n_reads = b->wro[d->n_windows];
  b->seq_off.assign(d->seq_off, d->seq_off + b->n_reads + 1);
  cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, dev);
  b->lmax.assign(b->n_windows, 1);
  b->sumlen.assign(b->n_windows, 0);
  b->nreads.assign(b->n_windows, 0);
  for (uint32_t w = 0; w < b->n_windows; ++w) {
    for (uint32_t r = b->wro[w]; r < b->wro[w + 1]; ++r) {
      uint64_t L = b->seq_off[r + 1] - b->seq_off[r];
      if (L > (uint64_t)INT32_MAX) {
        delete b;
        return kTooLarge;
      }
      b->lmax[w] = std::max<uint32_t>(b->lmax[w], (uint32_t)L);
      b->sumlen[w] += L;
    }
    b->nreads[w] = b->wro[w + 1] - b->wro[w];
  }
  // Per window: the lane width its reads are expected to need (the int16
  // rule of the reference evaluated against an estimate of the final graph,
  // L x (1 + reads / 10) nodes; a window that turns out to need int32 is
  // rerun with the int32 kernel) and the first graph capacity.  Windows are
  // then grouped into one pass per (width, tile) bucket, so short windows do
  // not run in the tile of the longest one; each pass is longest work first.
  {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
      cudaGetLastError();
      delete b;
      return kCuda;
    }
    b->budget = d->memory_budget ? d->memory_budget : (uint64_t)(free_b * 0.6);
  }
  b->plan0.assign(b->n_windows, WindowPlan{});
  for (uint32_t w = 0; w < b->n_windows; ++w) {
    const uint64_t est = std::min<uint64_t>(
        b->sumlen[w], (uint64_t)b->lmax[w] + (uint64_t)b->lmax[w] * b->nreads[w] / 10);
    b->plan0[w].wide = lanes_for(base, b->lmax[w], (uint32_t)std::min<uint64_t>(est, 0xFFFFFFFFu)) == 8;
    b->plan0[w].nodes =
        std::min<uint64_t>(std::max<uint64_t>(4096, 6ull * b->lmax[w] + 64), b->sumlen[w] + 1);
  }
  {
    std::vector<uint32_t> all(b->n_windows);
    for (uint32_t w = 0; w < b->n_windows; ++w) all[w] = w;
    st = make_passes(b, all, b->plan0, &b->passes);
    if (st) {
      delete b;
      return st;
    }
  }
  // first-pass consensus regions
  b->cons_off.assign(b->n_windows + 1, 0);
  for (uint32_t w = 0; w < b->n_windows; ++w)
    b->cons_off[w + 1] = b->cons_off[w] +
                         std::min<uint64_t>(b->sumlen[w] + 1, 2ull * b->lmax[w] + 64);
  cudaStream_t s = 0;
  const uint64_t nbytes = b->seq_off[b->n_reads];
  st = upload(b->d_seqs, reinterpret_cast<const uint8_t*>(d->seqs), nbytes, s);
  if (!st) st = upload(b->d_seq_off, b->seq_off.data(), b->seq_off.size(), s);
  if (!st && d->quals) st = upload(b->d_quals, reinterpret_cast<const uint8_t*>(d->quals), nbytes, s);
  if (!st) st = upload(b->d_wro, b->wro.data(), b->wro.size(), s);
  if (!st && d->window_type) st = upload(b->d_wtype, d->window_type, b->n_windows, s);
  if (!st && d->window_strand) st = upload(b->d_wstrand, d->window_strand, b->n_windows, s);
  if (!st) st = upload(b->d_cons_off, b->cons_off.data(), b->cons_off.size(), s);
  if (!st && (b->d_work.ensure(4ull * b->n_windows + 8) || b->d_cells.ensure(16) || b->d_queue.ensure(4ull * b->n_windows + 8) ||
              b->d_scores.ensure(4ull * b->n_reads + 8) || b->d_rev.ensure(b->n_reads + 8) ||
              b->d_cons.ensure(b->cons_off[b->n_windows] + 8) ||
              b->d_cons_len.ensure(4ull * b->n_windows + 8) ||
              b->d_status.ensure(4ull * b->n_windows + 8) || b->d_cells.ensure(8)))
    st = kNoMemory;
  if (!st && d->want_alignments) {
    b->aln_off.assign(b->n_reads + 1, 0);
    for (uint32_t w = 0; w < b->n_windows; ++w)
      for (uint32_t r = b->wro[w]; r < b->wro[w + 1]; ++r)
        b->aln_off[r + 1] = b->aln_off[r] + b->sumlen[w] + (b->seq_off[r + 1] - b->seq_off[r]) + 16;
    st = upload(b->d_aln_off, b->aln_off.data(), b->aln_off.size(), s);
    if (!st && (b->d_aln.ensure(8 * b->aln_off[b->n_reads] + 8) ||
                b->d_aln_len.ensure(4ull * b->n_reads + 8)))
      st = kNoMemory;
  }
  if (!st && d->want_msa) {
    b->msa_off.assign(b->n_windows + 1, 0);
    for (uint32_t w = 0; w < b->n_windows; ++w)
      b->msa_off[w + 1] = b->msa_off[w] + (uint64_t)(b->nreads[w] + 1) * (b->sumlen[w] + 1);
    st = upload(b->d_msa_off, b->msa_off.data(), b->msa_off.size(), s);
    if (!st && (b->d_msa.ensure(b->msa_off[b->n_windows] + 8) ||
                b->d_msa_rows.ensure(4ull * b->n_windows + 8) ||
                b->d_msa_cols.ensure(4ull * b->n_windows + 8)))
      st = kNoMemory;
  }
  if (!st && cudaStreamSynchronize(s) != cudaSuccess) st = kCuda;
  if (st) {
    cudaGetLastError();
    delete b;
    return st;
  }
  *out = b;
  return kOk;
}

int32_t spoa_gb300_batch_launch(spoa_gb300_batch* b, void* stream) {
  if (!b) return kInvalidArgument;
  if (!b->n_windows) return kOk;
  DeviceGuard guard(b->device);
  if (!guard.ok) return kCuda;
  return launch_all(b, stream, false);
}

int32_t spoa_gb300_batch_launch_plain(spoa_gb300_batch* b, void* stream) {
  if (!b) return kInvalidArgument;
  if (!b->n_windows) return kOk;
  DeviceGuard guard(b->device);
  if (!guard.ok) return kCuda;
  return launch_all(b, stream, true);
}

int32_t spoa_gb300_batch_fetch(spoa_gb300_batch* b, spoa_gb300_batch_result* r) {
  if (!b || !r) return kInvalidArgument;
  DeviceGuard guard(b->device);
  if (!guard.ok) return kCuda;
  std::memset(r, 0, sizeof(*r));
  const uint32_t W = b->n_windows, R = b->n_reads;
  b->h_scores.resize(R + 1);
  b->h_rev.resize(R + 1);
  b->h_status.resize(W + 1);
  std::vector<uint32_t> lens(W + 1);
  std::vector<char> raw(b->cons_off[W] + 1);
  uint64_t cells2[2] = {0, 0};
  if (R) {
    CU(cudaMemcpy(b->h_scores.data(), b->d_scores.p, 4ull * R, cudaMemcpyDeviceToHost));
    CU(cudaMemcpy(b->h_rev.data(), b->d_rev.p, R, cudaMemcpyDeviceToHost));
  }
  if (W) {
    CU(cudaMemcpy(b->h_status.data(), b->d_status.p, 4ull * W, cudaMemcpyDeviceToHost));
    CU(cudaMemcpy(lens.data(), b->d_cons_len.p, 4ull * W, cudaMemcpyDeviceToHost));
    CU(cudaMemcpy(raw.data(), b->d_cons.p, b->cons_off[W], cudaMemcpyDeviceToHost));
  }
  CU(cudaMemcpy(cells2, b->d_cells.p, 16, cudaMemcpyDeviceToHost));
  b->h_cons.clear();
  b->h_cons_off.assign(W + 1, 0);
  for (uint32_t w = 0; w < W; ++w) {
    if (b->h_status[w] == kOk) {
      if (w < b->retried.size() && b->retried[w]) {
        b->h_cons.insert(b->h_cons.end(), b->retry_cons[w].begin(), b->retry_cons[w].end());
      } else {
        uint64_t n = std::min<uint64_t>(lens[w], b->cons_off[w + 1] - b->cons_off[w]);
        b->h_cons.insert(b->h_cons.end(), raw.data() + b->cons_off[w], raw.data() + b->cons_off[w] + n);
      }
    }
    b->h_cons_off[w + 1] = b->h_cons.size();
  }
  b->h_cons.push_back(0);
  if (b->desc.want_alignments) {
    b->h_aln_len.resize(R + 1);
    if (R) CU(cudaMemcpy(b->h_aln_len.data(), b->d_aln_len.p, 4ull * R, cudaMemcpyDeviceToHost));
    std::vector<int32_t> all(2 * b->aln_off[R] + 2);
    if (R) CU(cudaMemcpy(all.data(), b->d_aln.p, 8 * b->aln_off[R], cudaMemcpyDeviceToHost));
    b->h_aln.clear();
    b->h_aln_off.assign(R + 1, 0);
    for (uint32_t k = 0; k < R; ++k) {
      uint64_t n = std::min<uint64_t>(b->h_aln_len[k], b->aln_off[k + 1] - b->aln_off[k]);
      b->h_aln.insert(b->h_aln.end(), all.begin() + 2 * b->aln_off[k],
                      all.begin() + 2 * (b->aln_off[k] + n));
      b->h_aln_off[k + 1] = b->h_aln_off[k] + n;
    }
    b->h_aln.push_back(0);
    r->alignments = b->h_aln.data();
    r->alignment_off = b->h_aln_off.data();
  }
  if (b->desc.want_msa) {
    b->h_msa.resize(b->msa_off[W] + 1);
    b->h_msa_rows.resize(W + 1);
    b->h_msa_cols.resize(W + 1);
    if (W) {
      CU(cudaMemcpy(b->h_msa.data(), b->d_msa.p, b->msa_off[W], cudaMemcpyDeviceToHost));
      CU(cudaMemcpy(b->h_msa_rows.data(), b->d_msa_rows.p, 4ull * W, cudaMemcpyDeviceToHost));
      CU(cudaMemcpy(b->h_msa_cols.data(), b->d_msa_cols.p, 4ull * W, cudaMemcpyDeviceToHost));
    }
    r->msa = b->h_msa.data();
    r->msa_off = b->msa_off.data();
    r->msa_rows = b->h_msa_rows.data();
    r->msa_cols = b->h_msa_cols.data();
  }
  r->read_scores = b->h_scores.data();
  r->read_reversed = b->h_rev.data();
  r->window_status = b->h_status.data();
  r->consensus = b->h_cons.data();
  r->consensus_off = b->h_cons_off.data();
  r->cells = cells2[0];
  r->pred_cells = cells2[1];
  r->kernel_ms = b->kernel_ms;
  // the tile of the pass with the most windows
  const Pass* big = nullptr;
  for (const Pass& p : b->passes)
    if (!big || p.windows.size() > big->windows.size()) big = &p;
  r->threads_per_window = big ? big->nt : 0;
  r->columns_per_thread = big ? big->cpt : 0;
  r->ctas = big ? big->ctas : 0;
  r->launches = b->launches;
  return kOk;
}

void spoa_gb300_batch_destroy(spoa_gb300_batch* b) {
  if (!b) return;
  DeviceGuard guard(b->device);
  delete b;
}

int32_t spoa_gb300_batch_run(const spoa_gb300_batch_desc* d, spoa_gb300_batch** out,
                             spoa_gb300_batch_result* r) {
  int32_t st = spoa_gb300_batch_create(d, out);
  if (st) return st;
  st = spoa_gb300_batch_launch(*out, nullptr);
  if (st) return st;
  return spoa_gb300_batch_fetch(*out, r);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// one window without device allocation
// ---------------------------------------------------------------------------
// Callers that must not allocate device memory (code that runs between the
// captures of a CUDA graph, allocators that own every byte of the device, or
// latency-critical loops that cannot afford cudaMalloc's implicit
// synchronisation) run a window through the same persistent kernel with its
// arena in this file-scope array.  Every device that loads the library holds
// it until the process exits.  All calls share it, so calls that overlap on
// the GPU race with each other.
namespace {

constexpr uint64_t kNoAllocBytes = SPOA_GB300_NOALLOC_SCRATCH_BYTES;
static __device__ __align__(256) uint8_t g_noalloc_scratch[kNoAllocBytes];

// bookkeeping of the batch kernel at the start of the array
struct NoAllocHeader {
  uint32_t queue;                  // work-queue cursor, must start at 0
  uint32_t work[1];                // the one window
  uint32_t win_read_off[2];        // {0, n_reads}
  int8_t strand[4];                // strand-ambiguous flag of the window
  uint64_t cons_off[2];            // {0, consensus capacity}
  unsigned long long cells[2];     // cell counters, must start at 0
  int32_t scores[SPOA_GB300_NOALLOC_MAX_READS];
  uint8_t reversed[SPOA_GB300_NOALLOC_MAX_READS];
};

__global__ void k_noalloc_setup(NoAllocHeader* h, uint32_t n_reads, uint64_t cons_cap,
                                int32_t strand) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  h->queue = 0;
  h->strand[0] = strand ? 1 : 0;
  h->work[0] = 0;
  h->win_read_off[0] = 0;
  h->win_read_off[1] = n_reads;
  h->cons_off[0] = 0;
  h->cons_off[1] = cons_cap;
  h->cells[0] = h->cells[1] = 0;
}

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[256] = {};

// Device address of the array for the current device, looked up once per
// device (the host-side name is only a stand-in for it).
int32_t noalloc_scratch(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) {
    cudaGetLastError();
    return kCuda;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
      cudaGetLastError();
      return kCuda;
    }
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return kOk;
}

}  // namespace

extern "C" int32_t spoa_gb300_window_poa_noalloc(
    int32_t type, int8_t m, int8_t n, int8_t g, int8_t e, int8_t q, int8_t c,
    int32_t strand_ambiguous, uint32_t n_reads, uint32_t max_read_len, const char* d_seqs,
    const uint64_t* d_seq_off, const char* d_quals, char* d_consensus, uint32_t consensus_cap,
    uint32_t* d_consensus_len, int32_t* d_read_scores, int32_t* d_status, void* stream) {
  if (type != kSW && type != kNW && type != kOV) return kInvalidArgument;
  if (g > 0 || q > 0 || e > 0 || c > 0) return kInvalidArgument;
  if (!d_seqs || !d_seq_off || !d_consensus || !d_consensus_len || !d_status || n_reads == 0)
    return kInvalidArgument;
  if (n_reads > SPOA_GB300_NOALLOC_MAX_READS || max_read_len > SPOA_GB300_NOALLOC_MAX_READ_LEN ||
      max_read_len == 0)
    return kTooLarge;
  const int32_t sub = g >= e ? kLinear : ((g <= q || e >= c) ? kAffine : kConvex);
  if (sub == kLinear) {
    e = g;
  } else if (sub == kAffine) {
    q = g;
    c = e;
  }
  int cpt = 0, nt = 0;
  if (!throughput_tile(max_read_len, false, &cpt, &nt)) return kTooLarge;
  GraphCaps gc;
  gc.nodes = SPOA_GB300_NOALLOC_MAX_NODES;
  gc.edges = 4 * SPOA_GB300_NOALLOC_MAX_NODES + 64;
  gc.labels = SPOA_GB300_NOALLOC_MAX_READS * SPOA_GB300_NOALLOC_MAX_READ_LEN + 2;
  gc.seqs = n_reads + 1;
  gc.aligned = SPOA_GB300_NOALLOC_MAX_ALIGNED;
  DpCaps dc{gc.nodes + 1, (uint32_t)(cpt * nt), gc.edges + gc.nodes + 2, sub, 2};  // int16 only
  GraphView gv;
  DpView dv;
  const uint64_t head = align_up(sizeof(NoAllocHeader), 256);
  const uint64_t gbytes = align_up(graph_layout(nullptr, gc, &gv), 256);
  const uint64_t dbytes = align_up(dp_layout(nullptr, dc, &dv), 256);
  if (head + gbytes + dbytes > kNoAllocBytes) return kTooLarge;
  void* scratch = nullptr;
  int32_t st = noalloc_scratch(&scratch);
  if (st) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  NoAllocHeader* h = static_cast<NoAllocHeader*>(scratch);
  k_noalloc_setup<<<1, 32, 0, s>>>(h, n_reads, consensus_cap, strand_ambiguous);
  CU(cudaGetLastError());
  BatchArgs a{};
  a.base = Scoring{type, sub, m, n, g, e, q, c};
  a.win_type = nullptr;
  a.win_strand = strand_ambiguous ? h->strand : nullptr;
  a.n_windows = 1;
  a.win_read_off = h->win_read_off;
  a.seqs = reinterpret_cast<const uint8_t*>(d_seqs);
  a.seq_off = d_seq_off;
  a.quals = reinterpret_cast<const uint8_t*>(d_quals);
  a.work = h->work;
  a.n_work = 1;
  a.queue = &h->queue;
  a.arena = static_cast<uint8_t*>(scratch) + head;
  a.arena_stride = gbytes + dbytes;
  a.gcaps = gc;
  a.dcaps = dc;
  a.read_scores = d_read_scores ? d_read_scores : h->scores;
  a.read_rev = h->reversed;
  a.cons = reinterpret_cast<uint8_t*>(d_consensus);
  a.cons_off = h->cons_off;
  a.cons_len = d_consensus_len;
  a.win_status = d_status;
  a.cells = &h->cells[0];
  a.pred_cells = &h->cells[1];
  return SPOA_BY_SUB(sub, false, launch_batch, cpt, nt, 1, a, s);
}

// ===========================================================================
// served windows: continuous batching
// ===========================================================================
namespace {

using Clock = std::chrono::steady_clock;

// First-fit allocator over one device region (the admission budget): a
// launch is admitted only when its whole footprint fits.
class DevicePool {
 public:
  int32_t init(uint64_t bytes) {
    if (cudaMalloc(&base_, bytes) != cudaSuccess) {
      cudaGetLastError();
      base_ = nullptr;
      return kNoMemory;
    }
    size_ = bytes;
    free_[0] = bytes;
    return kOk;
  }
  ~DevicePool() {
    if (base_) cudaFree(base_);
  }
  // offset of a free block of `bytes` (256-aligned), or ~0ull
  uint64_t alloc(uint64_t bytes) {
    bytes = align_up(std::max<uint64_t>(bytes, 256), 256);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second < bytes) continue;
      const uint64_t off = it->first, len = it->second;
      free_.erase(it);
      if (len > bytes) free_[off + bytes] = len - bytes;
      used_[off] = bytes;
      return off;
    }
    return ~0ull;
  }
  void release(uint64_t off) {
    auto u = used_.find(off);
    if (u == used_.end()) return;
    uint64_t len = u->second;
    used_.erase(u);
    auto next = free_.lower_bound(off);
    if (next != free_.end() && off + len == next->first) {
      len += next->second;
      next = free_.erase(next);
    }
    if (next != free_.begin()) {
      auto prev = std::prev(next);
      if (prev->first + prev->second == off) {
        prev->second += len;
        return;
      }
    }
    free_[off] = len;
  }
  uint8_t* ptr(uint64_t off) const { return static_cast<uint8_t*>(base_) + off; }
  uint64_t size() const { return size_; }

 private:
  void* base_ = nullptr;
  uint64_t size_ = 0;
  std::map<uint64_t, uint64_t> free_, used_;
};

// One submitted window.
struct ServedWindow {
  uint64_t ticket = 0;
  std::string seqs;
  std::vector<uint64_t> off;  // n_reads + 1
  int8_t type = 0, strand = 0;
  uint32_t lmax = 1;
  uint64_t sumlen = 0;
  WindowPlan plan;
  bool resident_failed = false;  // the resident kernel could not hold it
  Clock::time_point arrival;
  // results
  bool done = false;
  int32_t status = kOk;
  std::string consensus;
  Clock::time_point finished;
};

// Pinned staging buffers are allocated when the server starts and grow
// geometrically (from kPinnedMin), so serving rarely calls the page-locked
// allocator, which is slow and an implicit synchronisation point.
constexpr uint64_t kPinnedMin = 1ull << 20;
bool grow_pinned(uint8_t*& p, uint64_t& cap, uint64_t need) {
  if (p != nullptr && cap >= need) return true;
  const uint64_t want = std::max(std::max(need, 2 * cap), kPinnedMin);
  if (p) cudaFreeHost(p);
  p = nullptr;
  cap = 0;
  if (cudaHostAlloc(&p, want, cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();
    p = nullptr;
    return false;
  }
  cap = want;
  return true;
}

// One launch in flight: its windows, its block of the pool, its pinned
// staging buffer and the offsets of the parts inside both.
struct ServedLaunch {
  std::vector<std::shared_ptr<ServedWindow>> windows;
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  uint64_t pool_off = ~0ull;
  uint8_t* pinned = nullptr;
  uint64_t pinned_cap = 0;
  uint64_t in_bytes = 0, out_off = 0, out_bytes = 0;
  uint64_t o_cons_off = 0, o_cons = 0, o_cons_len = 0, o_status = 0;
  std::vector<uint64_t> cons_off;
  bool busy = false;
};

// The resident form of the server: polishing-sized windows (16-bit
// scores, reads of at most 640 bases) go to one persistent kernel (k_serve)
// that keeps running while work keeps arriving.  Each window takes a slot of
// a ring in host-mapped memory; its reads are copied to the device in
// batches, and a batch is published (ring slots filled, `tail` raised)
// once its copy has completed.  The kernel's CTAs claim published slots and
// write each consensus and status back into host-mapped memory.
constexpr uint32_t kResidentMaxLen = 640;  // one warp of 20 columns per thread
constexpr uint32_t kResidentMaxReads = 255;
constexpr uint64_t kResidentMaxBases = 65534;
constexpr uint32_t kResidentRing = 8192;
constexpr uint32_t kResidentConsCap = 2 * kResidentMaxLen + 64;
constexpr unsigned long long kResidentIdleNs = 20ull * 1000 * 1000;  // 20 ms without work

struct ResidentStage {  // one batch of windows on its way to the device
  uint8_t* pinned = nullptr;
  uint64_t cap = 0;
  cudaEvent_t copied = nullptr;
  std::vector<uint64_t> ks;  // ring slots of the batch, in order
};

struct Resident {
  bool ready = false;
  bool failed = false;  // set-up failed: the launch path serves every window
  int cpt = 0, nt = 0, ctas = 0;
  GraphCaps gc{};
  DpCaps dc{};
  uint64_t stride = 0, arena_off = ~0ull;
  void* host = nullptr;  // the mapped block: ring, done, tail, consensus
  ptrdiff_t host_to_dev = 0;  // device address of the mapped block minus its host address
  ServeSlot* ring = nullptr;
  ServeDone* done = nullptr;
  unsigned long long* tail = nullptr;
  uint8_t* cons = nullptr;
  DeviceBuf head;
  cudaStream_t stream = nullptr;
  cudaEvent_t ended = nullptr;
  bool launched = false;
  uint64_t next = 0, published = 0, head_seen = 0;
  struct Entry {
    std::shared_ptr<ServedWindow> w;
    uint64_t in_off = ~0ull;
    bool live = false;
  };
  std::vector<Entry> entries;      // per ring slot
  std::deque<uint64_t> in_flight;  // published slots not yet finished
  std::deque<ResidentStage> staging;
  std::vector<ResidentStage> spare;
  std::atomic<uint64_t> windows{0}, launches{0};
  template <typename X>
  X* dev(X* host_ptr) const {
    return reinterpret_cast<X*>(reinterpret_cast<uint8_t*>(host_ptr) + host_to_dev);
  }
};

}  // namespace

struct spoa_gb300_server {
  spoa_gb300_server_desc desc{};
  Scoring base{};
  int device = 0;
  int sm_count = 1;
  DevicePool pool;
  Resident res;
  std::vector<ServedLaunch> slots;
  std::mutex mu;
  std::condition_variable cv;  // completions, for wait()
  std::multimap<Clock::time_point, std::shared_ptr<ServedWindow>> incoming;  // not yet arrived
  std::deque<std::shared_ptr<ServedWindow>> pending;  // arrived, waiting for admission
  std::unordered_map<uint64_t, std::shared_ptr<ServedWindow>> tickets;
  uint64_t next_ticket = 1;
  std::atomic<uint64_t> launches{0}, completed{0};
  std::atomic<bool> stop{false};
  std::thread loop;
};

namespace {

uint64_t a16(uint64_t x) { return align_up(x, 16); }

// Length class of a window: up to 640 columns, then doublings (the classes
// of the batched passes); windows of one launch share class and width.
int length_class(uint32_t lmax) {
  int cls = 0;
  for (uint64_t cap = 640; cap < lmax; cap *= 2) ++cls;
  return cls;
}

// Marks a window finished (under the lock) and wakes the waiters.
void finish_window(spoa_gb300_server* sv, const std::shared_ptr<ServedWindow>& w, int32_t status,
                   std::string consensus) {
  std::lock_guard<std::mutex> lk(sv->mu);
  w->status = status;
  w->consensus = std::move(consensus);
  w->finished = Clock::now();
  w->done = true;
  ++sv->completed;
  sv->cv.notify_all();
}

bool resident_eligible(const spoa_gb300_server* sv, const ServedWindow& w);


// Takes arrived windows of the front window's class and width (in arrival
// order) into a free slot while their footprint fits the pool; false when
// nothing could be admitted.
bool admit(spoa_gb300_server* sv, ServedLaunch& L) {
  std::vector<std::shared_ptr<ServedWindow>> take;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    // windows the resident kernel takes are not launched
    auto first = std::find_if(sv->pending.begin(), sv->pending.end(),
                              [&](const std::shared_ptr<ServedWindow>& w) {
                                return !resident_eligible(sv, *w);
                              });
    if (first == sv->pending.end()) return false;
    const auto& f = *first;
    const bool wide = f->plan.wide;
    const int cls = length_class(f->lmax);
    const size_t cap = (size_t)std::max(1, sv->desc.max_windows_per_launch);
    for (auto it = first; it != sv->pending.end() && take.size() < cap; ++it)
      if (!resident_eligible(sv, **it) && (*it)->plan.wide == wide &&
          length_class((*it)->lmax) == cls)
        take.push_back(*it);
  }
  const bool wide = take.front()->plan.wide;
  // footprint of the first k windows (arenas for the CTAs or clusters that
  // run them); halve k until it fits the pool
  size_t k = take.size();
  while (k > 0) {
    uint32_t lmax = 1, maxreads = 1;
    uint64_t maxsum = 1, nodes = 1, R = 0, S = 0;
    bool many = false;
    for (size_t i = 0; i < k; ++i) {
      const ServedWindow& w = *take[i];
      lmax = std::max(lmax, w.lmax);
      maxsum = std::max(maxsum, w.sumlen);
      maxreads = std::max<uint32_t>(maxreads, (uint32_t)(w.off.size() - 1));
      nodes = std::max(nodes, w.plan.nodes);
      many = many || w.plan.many_aligned;
      R += w.off.size() - 1;
      S += w.sumlen;
    }
    // the batched kernel's tiles: long 32-bit rows on thread-block clusters,
    // past their range the segmented forward
    int cpt = 0, nt = 0, segs = 1, cl = 1;
    bool tiled;
    if (wide && cluster_tile(lmax, k, sv->sm_count, 0, &cl, &nt)) {
      cpt = kClCpt;
      tiled = true;
    } else {
      tiled = wide && lmax > (uint32_t)kSegCpt * 512 ? seg_tile(lmax, &cpt, &nt, &segs)
                                                      : throughput_tile(lmax, wide, &cpt, &nt);
    }
    if (!tiled) {
      // a read longer than any tile: the window fails alone
      auto w = take.front();
      {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->pending.erase(std::find(sv->pending.begin(), sv->pending.end(), w));
      }
      finish_window(sv, w, kTooLarge, std::string());
      return true;
    }
    GraphCaps gc;
    DpCaps dc;
    const uint64_t stride =
        arena_caps(sv->base.sub, wide, cpt * segs * cl, nt, nodes, maxsum, maxreads, many, &gc,
                   &dc);
    // the kernels are persistent (every CTA, or cluster, takes windows from
    // the work queue until it is empty): launch no more than can be
    // resident at once
    int resident = 0;
    if ((cl > 1     ? SPOA_BY_SUB16(sv->base.sub, occupancy_batch_cl, cl, nt, &resident)
         : segs > 1 ? SPOA_BY_SUB32(sv->base.sub, occupancy_batch_seg, segs, nt, &resident)
                    : SPOA_BY_SUB(sv->base.sub, wide, occupancy_batch, cpt, nt, &resident)) != kOk)
      resident = 1;
    if (cl == 1) resident *= sv->sm_count;
    const uint64_t grid = std::min<uint64_t>(k, (uint64_t)std::max(resident, 1));
    // inputs: work, queue, window read offsets, read offsets, types, strands,
    // consensus offsets, reads; outputs: scores, strands, lengths, status,
    // cell counters, consensus; then the arenas
    const uint64_t n = k;
    uint64_t o = 0;
    const uint64_t i_work = o; o = a16(o + 4 * n);
    const uint64_t i_queue = o; o = a16(o + 16);
    const uint64_t i_wro = o; o = a16(o + 4 * (n + 1));
    const uint64_t i_soff = o; o = a16(o + 8 * (R + 1));
    const uint64_t i_type = o; o = a16(o + n);
    const uint64_t i_strand = o; o = a16(o + n);
    const uint64_t i_coff = o; o = a16(o + 8 * (n + 1));
    const uint64_t i_seqs = o; o = a16(o + S);
    const uint64_t in_bytes = o;
    const uint64_t o_scores = o; o = a16(o + 4 * R);
    const uint64_t o_rev = o; o = a16(o + R);
    const uint64_t o_clen = o; o = a16(o + 4 * n);
    const uint64_t o_status = o; o = a16(o + 4 * n);
    const uint64_t o_cells = o; o = a16(o + 16);
    const uint64_t o_cons = o; o = a16(o + S + n);
    const uint64_t arena_off = align_up(o, 256);
    const uint64_t total = arena_off + stride * grid;
    if (total > sv->pool.size()) {
      if (k == 1) {  // can never fit: fail it
        auto w = take.front();
        {
          std::lock_guard<std::mutex> lk(sv->mu);
          sv->pending.erase(std::find(sv->pending.begin(), sv->pending.end(), w));
        }
        finish_window(sv, w, kNoMemory, std::string());
        return true;
      }
      k /= 2;
      continue;
    }
    const uint64_t off = sv->pool.alloc(total);
    if (off == ~0ull) {
      if (k == 1) return false;  // wait for memory to free up
      k /= 2;
      continue;
    }
    // admitted: stage the inputs in the slot's pinned buffer
    if (!grow_pinned(L.pinned, L.pinned_cap, arena_off)) {
      sv->pool.release(off);
      return false;
    }
    uint8_t* h = L.pinned;
    auto* work = reinterpret_cast<uint32_t*>(h + i_work);
    auto* wro = reinterpret_cast<uint32_t*>(h + i_wro);
    auto* soff = reinterpret_cast<uint64_t*>(h + i_soff);
    auto* wtype = reinterpret_cast<int8_t*>(h + i_type);
    auto* wstr = reinterpret_cast<int8_t*>(h + i_strand);
    auto* coff = reinterpret_cast<uint64_t*>(h + i_coff);
    std::memset(h + i_queue, 0, 16);
    L.cons_off.assign(n + 1, 0);
    uint64_t r = 0, sb = 0;
    wro[0] = 0;
    soff[0] = 0;
    coff[0] = 0;
    for (uint64_t i = 0; i < n; ++i) {
      const ServedWindow& w = *take[i];
      work[i] = (uint32_t)i;
      wtype[i] = w.type;
      wstr[i] = w.strand;
      std::memcpy(h + i_seqs + sb, w.seqs.data(), w.sumlen);
      for (size_t j = 0; j + 1 < w.off.size(); ++j) soff[r + j + 1] = sb + w.off[j + 1];
      r += w.off.size() - 1;
      sb += w.sumlen;
      wro[i + 1] = (uint32_t)r;
      coff[i + 1] = coff[i] + w.sumlen + 1;
      L.cons_off[i + 1] = coff[i + 1];
    }
    uint8_t* d = sv->pool.ptr(off);
    BatchArgs a{};
    a.base = sv->base;
    a.win_type = reinterpret_cast<int8_t*>(d + i_type);
    a.win_strand = reinterpret_cast<int8_t*>(d + i_strand);
    a.n_windows = (uint32_t)n;
    a.win_read_off = reinterpret_cast<uint32_t*>(d + i_wro);
    a.seqs = d + i_seqs;
    a.seq_off = reinterpret_cast<uint64_t*>(d + i_soff);
    a.work = reinterpret_cast<uint32_t*>(d + i_work);
    a.n_work = (uint32_t)n;
    a.queue = reinterpret_cast<uint32_t*>(d + i_queue);
    a.arena = d + arena_off;
    a.arena_stride = stride;
    a.gcaps = gc;
    a.dcaps = dc;
    a.read_scores = reinterpret_cast<int32_t*>(d + o_scores);
    a.read_rev = d + o_rev;
    a.cons = d + o_cons;
    a.cons_off = reinterpret_cast<uint64_t*>(d + i_coff);
    a.cons_len = reinterpret_cast<uint32_t*>(d + o_clen);
    a.win_status = reinterpret_cast<int32_t*>(d + o_status);
    a.cells = reinterpret_cast<unsigned long long*>(d + o_cells);
    a.pred_cells = a.cells + 1;
    bool ok = cudaMemcpyAsync(d, h, in_bytes, cudaMemcpyHostToDevice, L.stream) == cudaSuccess &&
              cudaMemsetAsync(d + o_cells, 0, 16, L.stream) == cudaSuccess;
    if (ok)
      ok = (cl > 1 ? SPOA_BY_SUB16(sv->base.sub, launch_batch_cl, cl, nt, (int)grid, a, L.stream)
            : segs > 1
                ? SPOA_BY_SUB32(sv->base.sub, launch_batch_seg, segs, nt, (int)grid, a, L.stream)
                : SPOA_BY_SUB(sv->base.sub, wide, launch_batch, cpt, nt, (int)grid, a, L.stream))
           == kOk;
    if (ok)
      ok = cudaMemcpyAsync(h + o_scores, d + o_scores, arena_off - o_scores, cudaMemcpyDeviceToHost,
                           L.stream) == cudaSuccess &&
           cudaEventRecord(L.done, L.stream) == cudaSuccess;
    {
      std::lock_guard<std::mutex> lk(sv->mu);
      for (size_t i = 0; i < k; ++i)
        sv->pending.erase(std::find(sv->pending.begin(), sv->pending.end(), take[i]));
    }
    L.windows.assign(take.begin(), take.begin() + k);
    L.pool_off = off;
    L.out_off = o_scores;
    L.o_cons = o_cons;
    L.o_cons_len = o_clen;
    L.o_status = o_status;
    L.busy = true;
    ++sv->launches;
    if (!ok) {
      cudaGetLastError();
      cudaStreamSynchronize(L.stream);
      sv->pool.release(off);
      L.busy = false;
      for (auto& w : L.windows) finish_window(sv, w, kCuda, std::string());
      L.windows.clear();
    }
    return true;
  }
  return false;
}

// A launch completed: hand out the results, or send windows that need the
// int32 width or a bigger arena back to the front of the queue.
void complete(spoa_gb300_server* sv, ServedLaunch& L, bool ok) {
  const uint8_t* h = L.pinned;
  const auto* status = reinterpret_cast<const int32_t*>(h + L.o_status);
  const auto* clen = reinterpret_cast<const uint32_t*>(h + L.o_cons_len);
  std::vector<std::shared_ptr<ServedWindow>> again;
  for (size_t i = 0; i < L.windows.size(); ++i) {
    auto& w = L.windows[i];
    const int32_t st = ok ? status[i] : kCuda;
    if (st == kNeedWide && !w->plan.wide) {
      w->plan.wide = true;
      again.push_back(w);
    } else if (st == kCapacity && (w->plan.nodes < w->sumlen + 1 || !w->plan.many_aligned)) {
      w->plan.nodes = std::min<uint64_t>(2 * w->plan.nodes, w->sumlen + 1);
      w->plan.many_aligned = true;
      again.push_back(w);
    } else {
      std::string cons;
      if (st == kOk) {
        const uint64_t cap = L.cons_off[i + 1] - L.cons_off[i];
        cons.assign(reinterpret_cast<const char*>(h + L.o_cons + L.cons_off[i]),
                    std::min<uint64_t>(clen[i], cap));
      }
      finish_window(sv, w, st, std::move(cons));
    }
  }
  if (!again.empty()) {
    std::lock_guard<std::mutex> lk(sv->mu);
    for (auto it = again.rbegin(); it != again.rend(); ++it) sv->pending.push_front(*it);
  }
  sv->pool.release(L.pool_off);
  L.windows.clear();
  L.busy = false;
}

// Sets up the resident kernel's ring, arenas and stream (first use).
bool resident_setup_once(spoa_gb300_server* sv);
bool resident_setup(spoa_gb300_server* sv) {
  Resident& R = sv->res;
  if (R.ready) return true;
  if (R.failed) return false;
  if (!resident_setup_once(sv)) R.failed = true;
  return R.ready;
}

bool resident_setup_once(spoa_gb300_server* sv) {
  Resident& R = sv->res;
  if (!throughput_tile(kResidentMaxLen, false, &R.cpt, &R.nt)) return false;
  int blocks = 1;
  if (SPOA_BY_SUB(sv->base.sub, false, occupancy_serve, R.cpt, R.nt, &blocks)) return false;
  int sms = 1;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, sv->device);
  // three quarters of the CTA slots: launches of other windows share the GPU
  uint64_t ctas = std::max<uint64_t>(1, (uint64_t)sms * std::max(blocks, 1) * 3 / 4);
  R.gc.nodes = 4096;
  R.gc.edges = 4 * R.gc.nodes + 64;
  R.gc.labels = (uint32_t)kResidentMaxBases + 2;
  R.gc.seqs = kResidentMaxReads + 1;
  R.gc.aligned = 4;
  R.dc = DpCaps{R.gc.nodes + 1, (uint32_t)(R.cpt * R.nt), R.gc.edges + R.gc.nodes + 2,
                sv->base.sub, 2};
  GraphView gv;
  DpView dv;
  R.stride = align_up(graph_layout(nullptr, R.gc, &gv), 256) +
             align_up(dp_layout(nullptr, R.dc, &dv), 256);
  // at most half of the budget for the resident arenas
  ctas = std::min<uint64_t>(ctas, std::max<uint64_t>(1, sv->pool.size() / 2 / R.stride));
  R.arena_off = sv->pool.alloc(R.stride * ctas);
  if (R.arena_off == ~0ull) return false;
  R.ctas = (int)ctas;
  const uint64_t bytes = a16(sizeof(ServeSlot) * kResidentRing) +
                         a16(sizeof(ServeDone) * kResidentRing) + a16(sizeof(unsigned long long)) +
                         (uint64_t)kResidentConsCap * kResidentRing;
  if (cudaHostAlloc(&R.host, bytes, cudaHostAllocMapped) != cudaSuccess) {
    cudaGetLastError();
    R.host = nullptr;
    return false;
  }
  std::memset(R.host, 0, bytes);
  void* dev = nullptr;
  if (cudaHostGetDevicePointer(&dev, R.host, 0) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  R.host_to_dev = static_cast<uint8_t*>(dev) - static_cast<uint8_t*>(R.host);
  uint8_t* h = static_cast<uint8_t*>(R.host);
  R.ring = reinterpret_cast<ServeSlot*>(h);
  h += a16(sizeof(ServeSlot) * kResidentRing);
  R.done = reinterpret_cast<ServeDone*>(h);
  h += a16(sizeof(ServeDone) * kResidentRing);
  R.tail = reinterpret_cast<unsigned long long*>(h);
  h += a16(sizeof(unsigned long long));
  R.cons = h;
  if (R.head.ensure(8) || cudaMemset(R.head.p, 0, 8) != cudaSuccess ||
      cudaStreamCreateWithFlags(&R.stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&R.ended, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  R.entries.resize(kResidentRing);
  // staging batches ready before windows arrive (pinned allocations can
  // wait for the device's work in flight)
  for (int k = 0; k < 4; ++k) {
    ResidentStage st;
    const bool ok = cudaEventCreateWithFlags(&st.copied, cudaEventDisableTiming) == cudaSuccess &&
                    grow_pinned(st.pinned, st.cap, kPinnedMin);
    if (!ok) {
      cudaGetLastError();
      if (st.copied) cudaEventDestroy(st.copied);
      if (st.pinned) cudaFreeHost(st.pinned);
      return false;
    }
    R.spare.push_back(std::move(st));
  }
  R.ready = true;
  return true;
}

bool resident_eligible(const spoa_gb300_server* sv, const ServedWindow& w) {
  return sv->desc.resident && !sv->res.failed && !w.plan.wide && !w.plan.many_aligned && !w.resident_failed &&
         w.off.size() > 1 && w.lmax <= kResidentMaxLen && w.off.size() - 1 <= kResidentMaxReads &&
         w.sumlen <= kResidentMaxBases;
}

// Moves arrived resident-eligible windows into one staging batch (ring
// slots, device input memory from the pool, one copy); false when nothing
// moved.
bool resident_admit(spoa_gb300_server* sv) {
  Resident& R = sv->res;
  std::vector<std::shared_ptr<ServedWindow>> take;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    for (const auto& w : sv->pending)
      if (resident_eligible(sv, *w)) take.push_back(w);
  }
  if (take.empty() || !resident_setup(sv)) return false;
  ResidentStage st;
  if (!R.spare.empty()) {
    st = std::move(R.spare.back());
    R.spare.pop_back();
  } else if (cudaEventCreateWithFlags(&st.copied, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  st.ks.clear();
  // inputs of the batch: per window its read offsets, then its reads
  std::vector<std::pair<uint64_t, uint64_t>> parts;  // (pool offset, bytes)
  uint64_t total = 0;
  size_t n = 0;
  for (; n < take.size(); ++n) {
    const ServedWindow& w = *take[n];
    const uint64_t k = R.next + n;
    if (R.entries[k % kResidentRing].live) break;  // ring full
    const uint64_t bytes = a16(8 * w.off.size()) + a16(w.sumlen);
    const uint64_t off = sv->pool.alloc(bytes);
    if (off == ~0ull) break;  // no memory now: the rest waits
    parts.emplace_back(off, bytes);
    total += bytes;
  }
  if (n == 0) {
    R.spare.push_back(std::move(st));
    return false;
  }
  if (!grow_pinned(st.pinned, st.cap, total)) {
    for (auto& p : parts) sv->pool.release(p.first);
    R.spare.push_back(std::move(st));
    return false;
  }
  uint64_t o = 0;
  bool ok = true;
  for (size_t i = 0; i < n; ++i) {
    const ServedWindow& w = *take[i];
    uint8_t* dst = st.pinned + o;
    std::memcpy(dst, w.off.data(), 8 * w.off.size());
    std::memcpy(dst + a16(8 * w.off.size()), w.seqs.data(), w.sumlen);
    ok = ok && cudaMemcpyAsync(sv->pool.ptr(parts[i].first), dst, parts[i].second,
                               cudaMemcpyHostToDevice, R.stream) == cudaSuccess;
    o += parts[i].second;
    const uint64_t k = R.next++;
    Resident::Entry& e = R.entries[k % kResidentRing];
    e.w = take[i];
    e.in_off = parts[i].first;
    e.live = true;
    st.ks.push_back(k);
    ServeSlot& slot = R.ring[k % kResidentRing];
    slot.seqs = sv->pool.ptr(parts[i].first) + a16(8 * w.off.size());
    slot.seq_off = reinterpret_cast<const uint64_t*>(sv->pool.ptr(parts[i].first));
    slot.cons = R.dev(R.cons + (uint64_t)(k % kResidentRing) * kResidentConsCap);
    slot.n_reads = (uint32_t)(w.off.size() - 1);
    slot.cons_cap = kResidentConsCap;
    slot.type = w.type;
    slot.strand = w.strand;
  }
  ok = ok && cudaEventRecord(st.copied, R.stream) == cudaSuccess;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    for (size_t i = 0; i < n; ++i)
      sv->pending.erase(std::find(sv->pending.begin(), sv->pending.end(), take[i]));
  }
  if (!ok) cudaGetLastError();  // the batch is published and reported after its event
  R.staging.push_back(std::move(st));
  return true;
}

// Publishes staged batches whose copy completed (in order), starts the
// kernel when it is not running and published work is unclaimed, and
// hands out finished windows.  Returns true when anything happened; sets
// *busy when windows are still in flight.
bool resident_progress(spoa_gb300_server* sv, bool* busy) {
  Resident& R = sv->res;
  *busy = false;
  if (!R.ready) return false;
  bool progress = false;
  while (!R.staging.empty()) {
    ResidentStage& st = R.staging.front();
    const cudaError_t q = cudaEventQuery(st.copied);
    if (q == cudaErrorNotReady) break;
    if (q != cudaSuccess) cudaGetLastError();
    for (uint64_t k : st.ks) R.in_flight.push_back(k);
    R.published = st.ks.back() + 1;
    std::atomic_thread_fence(std::memory_order_release);
    reinterpret_cast<std::atomic<unsigned long long>*>(R.tail)->store(R.published,
                                                                      std::memory_order_release);
    R.spare.push_back(std::move(st));
    R.staging.pop_front();
    progress = true;
  }
  // the kernel: (re)started when it has ended and published work is unclaimed
  if (R.published > R.head_seen) {
    const bool running = R.launched && cudaEventQuery(R.ended) == cudaErrorNotReady;
    if (!running) {
      cudaGetLastError();
      unsigned long long head = 0;
      if (cudaMemcpy(&head, R.head.p, 8, cudaMemcpyDeviceToHost) == cudaSuccess)
        R.head_seen = head;
      else
        cudaGetLastError();
      if (R.head_seen < R.published) {
        ServeArgs a{};
        a.base = sv->base;
        a.ring = R.dev(R.ring);
        a.done = R.dev(R.done);
        a.cap = kResidentRing;
        a.tail = R.dev(R.tail);
        a.head = R.head.as<unsigned long long>();
        a.arena = sv->pool.ptr(R.arena_off);
        a.arena_stride = R.stride;
        a.gcaps = R.gc;
        a.dcaps = R.dc;
        a.idle_ns = kResidentIdleNs;
        if (SPOA_BY_SUB(sv->base.sub, false, launch_serve, R.cpt, R.nt, R.ctas, a, R.stream) ==
                kOk &&
            cudaEventRecord(R.ended, R.stream) == cudaSuccess) {
          R.launched = true;
          ++R.launches;
          ++sv->launches;
          progress = true;
        } else {
          cudaGetLastError();
        }
      }
    }
  }
  // finished windows
  for (size_t i = 0; i < R.in_flight.size();) {
    const uint64_t k = R.in_flight[i];
    ServeDone& d = R.done[k % kResidentRing];
    const unsigned long long seq =
        reinterpret_cast<std::atomic<unsigned long long>*>(&d.seq)->load(std::memory_order_acquire);
    if (seq != k + 1) {
      ++i;
      continue;
    }
    Resident::Entry& e = R.entries[k % kResidentRing];
    std::shared_ptr<ServedWindow> w = std::move(e.w);
    const int32_t status = d.status;
    const uint32_t len = d.cons_len;
    sv->pool.release(e.in_off);
    e.live = false;
    R.in_flight.erase(R.in_flight.begin() + (long)i);
    progress = true;
    ++R.windows;
    if (status == kNeedWide || status == kCapacity) {
      // outside the resident kernel's limits: the launch path runs it again
      w->resident_failed = true;
      if (status == kNeedWide) w->plan.wide = true;
      std::lock_guard<std::mutex> lk(sv->mu);
      sv->pending.push_front(w);
      continue;
    }
    std::string cons;
    if (status == kOk)
      cons.assign(reinterpret_cast<const char*>(R.cons + (uint64_t)(k % kResidentRing) *
                                                             kResidentConsCap),
                  std::min<uint32_t>(len, kResidentConsCap));
    finish_window(sv, w, status, std::move(cons));
  }
  *busy = !R.in_flight.empty() || !R.staging.empty();
  return progress;
}

void serve_loop(spoa_gb300_server* sv) {
  cudaSetDevice(sv->device);
  const auto gather = std::chrono::duration<double>(std::max(0.0, sv->desc.gather_seconds));
  while (true) {
    bool progress = false, in_flight = false;
    for (ServedLaunch& L : sv->slots) {
      if (!L.busy) continue;
      const cudaError_t q = cudaEventQuery(L.done);
      if (q == cudaErrorNotReady) {
        in_flight = true;
        continue;
      }
      if (q != cudaSuccess) cudaGetLastError();
      complete(sv, L, q == cudaSuccess);
      progress = true;
    }
    bool waiting;
    {
      std::lock_guard<std::mutex> lk(sv->mu);
      const auto now = Clock::now();
      while (!sv->incoming.empty() && sv->incoming.begin()->first <= now) {
        sv->pending.push_back(sv->incoming.begin()->second);
        sv->incoming.erase(sv->incoming.begin());
      }
    }
    if (sv->desc.resident) {
      if (resident_admit(sv)) progress = true;
      bool busy = false;
      if (resident_progress(sv, &busy)) progress = true;
      if (busy) in_flight = true;
    }
    {
      std::lock_guard<std::mutex> lk(sv->mu);
      waiting = !sv->pending.empty() || !sv->incoming.empty();
    }
    for (ServedLaunch& L : sv->slots) {
      if (L.busy) continue;
      bool go;
      {
        std::lock_guard<std::mutex> lk(sv->mu);
        go = !sv->pending.empty() &&
             (gather.count() <= 0 ||
              (int64_t)sv->pending.size() >= sv->desc.max_windows_per_launch ||
              Clock::now() - sv->pending.front()->arrival >= gather);
      }
      if (!go || !admit(sv, L)) break;
      progress = true;
      in_flight = true;
    }
    if (sv->stop && !in_flight && !waiting) break;
    if (!progress) std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
}

}  // namespace

extern "C" {

int32_t spoa_gb300_server_create(const spoa_gb300_server_desc* d, spoa_gb300_server** out) {
  if (!d || !out) return kInvalidArgument;
  *out = nullptr;
  spoa_gb300_engine* en = nullptr;
  int32_t st = spoa_gb300_engine_create(d->type, d->m, d->n, d->g, d->e, d->q, d->c, &en);
  if (st) return st;
  auto* sv = new (std::nothrow) spoa_gb300_server();
  if (!sv) {
    spoa_gb300_engine_destroy(en);
    return kNoMemory;
  }
  sv->base = en->S;
  spoa_gb300_engine_destroy(en);
  sv->desc = *d;
  if (sv->desc.max_streams <= 0) sv->desc.max_streams = 32;
  if (sv->desc.max_windows_per_launch <= 0) sv->desc.max_windows_per_launch = 4096;
  sv->device = resolve_device(d->device_set, d->device);
  if (sv->device < 0) {
    delete sv;
    return d->device_set ? kInvalidArgument : kCuda;
  }
  DeviceGuard guard(sv->device);
  if (!guard.ok) {
    delete sv;
    return kCuda;
  }
  if (cudaDeviceGetAttribute(&sv->sm_count, cudaDevAttrMultiProcessorCount, sv->device) !=
          cudaSuccess ||
      sv->sm_count < 1) {
    cudaGetLastError();
    sv->sm_count = 1;
  }
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
    cudaGetLastError();
    delete sv;
    return kCuda;
  }
  const uint64_t budget = d->memory_budget ? d->memory_budget : (uint64_t)(free_b * 0.4);
  if (budget > free_b || sv->pool.init(budget)) {
    delete sv;
    return kNoMemory;
  }
  sv->slots.resize(sv->desc.max_streams);
  for (ServedLaunch& L : sv->slots) {
    if (cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&L.done, cudaEventDisableTiming) != cudaSuccess ||
        !grow_pinned(L.pinned, L.pinned_cap, kPinnedMin)) {
      cudaGetLastError();
      spoa_gb300_server_destroy(sv);
      return kCuda;
    }
  }
  sv->loop = std::thread(serve_loop, sv);
  *out = sv;
  return kOk;
}

int32_t spoa_gb300_server_submit(spoa_gb300_server* sv, const char* seqs, const uint64_t* seq_off,
                                 uint32_t n_reads, int32_t type, int32_t strand, double delay,
                                 uint64_t* ticket) {
  if (!sv || !seq_off || !ticket || (n_reads && !seqs) || sv->stop) return kInvalidArgument;
  if (type == -1) type = sv->desc.type;
  if (type != kSW && type != kNW && type != kOV) return kInvalidArgument;
  auto w = std::make_shared<ServedWindow>();
  w->type = (int8_t)type;
  w->strand = strand ? 1 : 0;
  w->off.assign(seq_off, seq_off + n_reads + 1);
  for (uint32_t r = 0; r < n_reads; ++r) {
    if (w->off[r + 1] < w->off[r]) return kInvalidArgument;
    const uint64_t L = w->off[r + 1] - w->off[r];
    if (L > (uint64_t)INT32_MAX) return kTooLarge;
    w->lmax = std::max<uint32_t>(w->lmax, (uint32_t)L);
  }
  for (auto& o : w->off) o -= seq_off[0];
  w->sumlen = w->off[n_reads];
  w->seqs.assign(seqs ? seqs + seq_off[0] : "", w->sumlen);
  // the plan of the batched passes: width from the estimated final graph,
  // the first graph capacity
  const uint64_t est = std::min<uint64_t>(w->sumlen, (uint64_t)w->lmax + (uint64_t)w->lmax * n_reads / 10);
  w->plan.wide = lanes_for(sv->base, w->lmax, (uint32_t)std::min<uint64_t>(est, 0xFFFFFFFFu)) == 8;
  w->plan.nodes = std::min<uint64_t>(std::max<uint64_t>(4096, 6ull * w->lmax + 64), w->sumlen + 1);
  w->arrival = Clock::now() + std::chrono::duration_cast<Clock::duration>(
                                  std::chrono::duration<double>(std::max(0.0, delay)));
  std::lock_guard<std::mutex> lk(sv->mu);
  w->ticket = sv->next_ticket++;
  sv->tickets[w->ticket] = w;
  sv->incoming.emplace(w->arrival, w);
  *ticket = w->ticket;
  return kOk;
}

int32_t spoa_gb300_server_wait(spoa_gb300_server* sv, uint64_t ticket, double timeout,
                               char* consensus, uint32_t cap, uint32_t* len, int32_t* status,
                               double* latency) {
  if (!sv) return kInvalidArgument;
  std::unique_lock<std::mutex> lk(sv->mu);
  auto it = sv->tickets.find(ticket);
  if (it == sv->tickets.end()) return kInvalidArgument;
  std::shared_ptr<ServedWindow> w = it->second;
  auto ready = [&] { return w->done; };
  if (timeout > 0) {
    if (!sv->cv.wait_for(lk, std::chrono::duration<double>(timeout), ready))
      return SPOA_GB300_ERR_TIMEOUT;
  } else {
    sv->cv.wait(lk, ready);
  }
  sv->tickets.erase(it);
  if (status) *status = w->status;
  if (len) *len = (uint32_t)w->consensus.size();
  if (consensus && cap) std::memcpy(consensus, w->consensus.data(), std::min<size_t>(cap, w->consensus.size()));
  if (latency) *latency = std::chrono::duration<double>(w->finished - w->arrival).count();
  return kOk;
}

int32_t spoa_gb300_server_stats(const spoa_gb300_server* sv, uint64_t* launches,
                                uint64_t* completed) {
  if (!sv) return kInvalidArgument;
  if (launches) *launches = sv->launches;
  if (completed) *completed = sv->completed;
  return kOk;
}

int32_t spoa_gb300_server_resident_stats(const spoa_gb300_server* sv, uint64_t* windows,
                                         uint64_t* launches) {
  if (!sv) return kInvalidArgument;
  if (windows) *windows = sv->res.windows;
  if (launches) *launches = sv->res.launches;
  return kOk;
}

void spoa_gb300_server_destroy(spoa_gb300_server* sv) {
  if (!sv) return;
  sv->stop = true;
  if (sv->loop.joinable()) sv->loop.join();
  DeviceGuard guard(sv->device);
  if (sv->res.ready) {
    cudaStreamSynchronize(sv->res.stream);
    for (auto* v : {&sv->res.staging}) {
      for (auto& st : *v) {
        if (st.pinned) cudaFreeHost(st.pinned);
        if (st.copied) cudaEventDestroy(st.copied);
      }
    }
    for (auto& st : sv->res.spare) {
      if (st.pinned) cudaFreeHost(st.pinned);
      if (st.copied) cudaEventDestroy(st.copied);
    }
  }
  if (sv->res.ended) cudaEventDestroy(sv->res.ended);
  if (sv->res.stream) cudaStreamDestroy(sv->res.stream);
  if (sv->res.host) cudaFreeHost(sv->res.host);
  for (ServedLaunch& L : sv->slots) {
    if (L.stream) cudaStreamDestroy(L.stream);
    if (L.done) cudaEventDestroy(L.done);
    if (L.pinned) cudaFreeHost(L.pinned);
  }
  delete sv;
}

}  // extern "C"
