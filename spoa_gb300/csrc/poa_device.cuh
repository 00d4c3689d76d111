// poa_device.cuh - device-resident POA window: graph, DP, traceback,
// consensus and MSA for one window, run by one CTA.
//
// A window is one spoa::Graph plus the per-read state of an AlignmentEngine.
// Everything a read needs (graph arrays, DP matrices, traceback buffers)
// lives in HBM in one arena per CTA; the graph never leaves the device
// between reads.
//
// Reference correspondence (spoa v4):
//   dp_forward / select / traceback  <- SimdAlignmentEngine::Linear/Affine/
//        Convex (src/simd_alignment_engine_implementation.hpp:782-2131)
//   width rule                       <- implementation.hpp:719-726 with
//        AlignmentEngine::WorstCaseAlignmentScore (alignment_engine.cpp:101)
//   g_add_alignment                  <- Graph::AddAlignment (graph.cpp:155)
//   g_topo_sort                      <- Graph::TopologicalSort (graph.cpp:249)
//   g_consensus                      <- TraverseHeaviestBundle/BranchCompletion
//                                       (graph.cpp:433-516)
//   g_msa                            <- GenerateMultipleSequenceAlignment
//                                       (graph.cpp:321-366)
#pragma once

#include <cstdint>

namespace spoa_gb300 {

constexpr uint32_t kNone = 0xFFFFFFFFu;
// Internal -infinity for row 0 of F/O.  The reference uses INT16_MIN+1024 or
// INT32_MIN+1024; the width rule keeps every reachable score above either,
// so row 0 of F/O never wins a max nor matches a traceback equality, and
// any value far below the reachable range gives identical results.
constexpr int32_t kNegBig = -(1 << 28);

enum Status : int32_t {
  kOk = 0,
  kInvalidArgument = 1,
  kTooLarge = 2,
  kOverflow = 3,
  kNoMemory = 4,
  kInvalidAlignment = 5,
  kMissingSequence = 6,
  kUnequalWeights = 7,
  kCapacity = 8,
  kTraceback = 9,
  kCuda = 10,
  kNeedWide = 11,  // internal: the window needs the int32 kernel
};

enum : int32_t { kSW = 0, kNW = 1, kOV = 2 };
enum : int32_t { kLinear = 0, kAffine = 1, kConvex = 2 };

struct Scoring {
  int32_t type, sub;
  int32_t m, n, g, e, q, c;
  // INT16_MIN in both 16-bit lanes.  Read from memory at run time so the
  // compiler cannot fold it: max3(a, b, min16x2) is one DPX instruction,
  // while a two-input 16x2 max compiles to a slower sequence.
  uint32_t min16x2 = 0x80008000u;
};

__host__ __device__ inline uint64_t align_up(uint64_t x, uint64_t a) {
  return (x + a - 1) / a * a;
}

// Host builds of the device code for the tests may define
// SPOA_GB300_HOST_REDZONE (with AddressSanitizer): every region of an arena
// is then followed by a poisoned red zone, so that an access past the end
// of a region is reported.  Device builds never define it.
#if defined(SPOA_GB300_HOST_REDZONE) && !defined(__CUDA_ARCH__)
#include <sanitizer/asan_interface.h>
#define SPOA_GB300_REDZONE(base, p, bytes, off)                                       \
  do {                                                                                \
    (off) += 256;                                                                     \
    if (base) ASAN_POISON_MEMORY_REGION((p) + (bytes), (base) + (off) - ((p) + (bytes))); \
  } while (0)
#else
#define SPOA_GB300_REDZONE(base, p, bytes, off) ((void)0)
#endif

// ---------------------------------------------------------------------------
// graph arena
// ---------------------------------------------------------------------------
struct GraphCaps {
  uint32_t nodes, edges, labels, seqs, aligned;  // aligned: per-node slots
};

struct GraphHeader {
  uint32_t n_nodes, n_edges, n_labels, n_seqs, num_codes, n_consensus;
  int32_t status;
  uint32_t pad;
  int32_t coder[256];
  int32_t decoder[256];
};

struct GraphView {
  GraphHeader* hdr;
  uint8_t* code;
  // per node: x = first in-edge, y = last in-edge, z = first out-edge,
  // w = last out-edge (edge lists in insertion order); one line per node
  uint4* nlink;
  uint32_t* in_deg;
  uint8_t* n_aligned;
  uint32_t* aligned;  // [nodes * caps.aligned]
  // per node: x = in-degree | aligned count << 16, y/z/w = the first three
  // in-edge tails in insertion order (one 16-byte load per DFS step)
  uint4* nrec;
  uint32_t *rank_to_node, *node_to_rank;
  // per edge: x = tail, y = head, z = next in-edge of the head, w = next
  // out-edge of the tail; one 16-byte load per step of a list walk
  uint4* erec;
  uint32_t *e_lab_first, *e_lab_last;
  int64_t* e_weight;
  uint32_t *lab_seq, *lab_next;
  uint32_t* seq_begin;
  uint32_t* consensus;
  // DFS state of the topological sort: per 32 nodes three words (in
  // progress, done, ignored), interleaved so one node's bits share a line
  uint32_t* sort_bits;
  uint32_t* stack;
  int64_t* cscore;
  uint32_t *cpred, *column;
  GraphCaps caps;
  uint64_t stack_cap;
};

// Lays out a graph arena at `base` (nullptr: only measure).  Returns bytes.
__host__ __device__ inline uint64_t graph_layout(uint8_t* base, const GraphCaps& c,
                                                 GraphView* v) {
  uint64_t off = 0;
  auto take = [&](uint64_t bytes) -> uint8_t* {
    uint8_t* p = base ? base + off : nullptr;
    off = align_up(off + bytes, 256);
    SPOA_GB300_REDZONE(base, p, bytes, off);
    return p;
  };
  const uint64_t N = c.nodes, E = c.edges;
  v->caps = c;
  v->stack_cap = E + N * (uint64_t)(c.aligned + 1) + 1;
  v->hdr = reinterpret_cast<GraphHeader*>(take(sizeof(GraphHeader)));
  v->code = take(N);
  v->nlink = reinterpret_cast<uint4*>(take(16 * N));
  v->in_deg = reinterpret_cast<uint32_t*>(take(4 * N));
  v->n_aligned = take(N);
  v->aligned = reinterpret_cast<uint32_t*>(take(4 * N * c.aligned));
  v->nrec = reinterpret_cast<uint4*>(take(16 * N));
  v->rank_to_node = reinterpret_cast<uint32_t*>(take(4 * N));
  v->node_to_rank = reinterpret_cast<uint32_t*>(take(4 * N));
  v->erec = reinterpret_cast<uint4*>(take(16 * E));
  v->e_lab_first = reinterpret_cast<uint32_t*>(take(4 * E));
  v->e_lab_last = reinterpret_cast<uint32_t*>(take(4 * E));
  v->e_weight = reinterpret_cast<int64_t*>(take(8 * E));
  v->lab_seq = reinterpret_cast<uint32_t*>(take(4 * (uint64_t)c.labels));
  v->lab_next = reinterpret_cast<uint32_t*>(take(4 * (uint64_t)c.labels));
  v->seq_begin = reinterpret_cast<uint32_t*>(take(4 * (uint64_t)c.seqs));
  v->consensus = reinterpret_cast<uint32_t*>(take(4 * N));
  v->sort_bits = reinterpret_cast<uint32_t*>(take(12 * ((N + 31) / 32)));
  v->stack = reinterpret_cast<uint32_t*>(take(4 * v->stack_cap));
  v->cscore = reinterpret_cast<int64_t*>(take(8 * N));
  v->cpred = reinterpret_cast<uint32_t*>(take(4 * N));
  v->column = reinterpret_cast<uint32_t*>(take(4 * N));
  return off;
}

// ---------------------------------------------------------------------------
// DP arena (per alignment engine / per CTA)
// ---------------------------------------------------------------------------
struct DpCaps {
  uint32_t rows;  // graph nodes + 1
  uint32_t ld;    // columns (>= threads * columns-per-thread)
  uint32_t preds; // in-edges + rows
  int32_t sub;
  int32_t esize = 4;  // bytes per DP element: 2 when only int16 kernels use it
};

struct DpView {
  // H/F/O rows in "pair layout": thread t's strip of CPT columns is held as
  // CPT/2 pairs, pair k = (column t*CPT + k, column t*CPT + CPT/2 + k), one
  // pair per 32-bit word (int16 lanes) or per 64-bit word (int32 lanes).
  // Pair k of thread t (of nt) is pair word (k/2)*2*nt + 2*t + k%2 of the
  // row, so pairs k, k+1 of all threads are contiguous and every row access
  // of the forward pass is a fully coalesced warp access (colmap<CPT>).
  // Elements are caps.esize bytes (2 for arenas only int16 kernels use).
  // H, F (affine, convex), O (convex) and the in-row gap rows E (affine,
  // convex) and Q (convex) as the recurrences computed them
  void *H, *F, *O, *E, *Q;
  uint32_t *pred_ptr, *preds, *row_indeg;
  uint8_t *row_char, *row_sink;
  // per row, what the forward pass needs in one 16-byte load: x = first
  // predecessor entry, y = predecessor count (saturated at 0xFFFF) |
  // flags << 16 | character << 24,
  // z / w = the first two predecessors other than the previous row (kNone
  // when absent)
  uint4* rowrec;
  int32_t *fc, *fcF, *fcO;
  int32_t *aln_a, *aln_b;  // traceback outputs, 2 ints per pair
  uint8_t* seq_rc;         // reverse complement / staging of the read
  DpCaps caps;
  uint64_t aln_cap;        // pairs
};

__host__ __device__ inline uint64_t dp_layout(uint8_t* base, const DpCaps& c, DpView* v) {
  uint64_t off = 0;
  auto take = [&](uint64_t bytes) -> uint8_t* {
    uint8_t* p = base ? base + off : nullptr;
    off = align_up(off + bytes, 256);
    SPOA_GB300_REDZONE(base, p, bytes, off);
    return p;
  };
  const uint64_t cells = (uint64_t)c.rows * c.ld;
  v->caps = c;
  v->aln_cap = (uint64_t)c.rows + c.ld + 16;
  const uint64_t mbytes = (uint64_t)c.esize * cells;
  v->H = take(mbytes);
  v->F = c.sub >= kAffine ? take(mbytes) : nullptr;
  v->O = c.sub == kConvex ? take(mbytes) : nullptr;
  v->E = c.sub >= kAffine ? take(mbytes) : nullptr;
  v->Q = c.sub == kConvex ? take(mbytes) : nullptr;
  v->pred_ptr = reinterpret_cast<uint32_t*>(take(4 * ((uint64_t)c.rows + 1)));
  v->preds = reinterpret_cast<uint32_t*>(take(4 * (uint64_t)c.preds));
  v->row_indeg = reinterpret_cast<uint32_t*>(take(4 * (uint64_t)c.rows));
  v->row_char = take(c.rows);
  v->row_sink = take(c.rows);
  v->rowrec = reinterpret_cast<uint4*>(take(16 * (uint64_t)c.rows));
  v->fc = reinterpret_cast<int32_t*>(take(4 * (uint64_t)c.rows));
  v->fcF = reinterpret_cast<int32_t*>(take(4 * (uint64_t)c.rows));
  v->fcO = reinterpret_cast<int32_t*>(take(4 * (uint64_t)c.rows));
  v->aln_a = reinterpret_cast<int32_t*>(take(8 * v->aln_cap));
  v->aln_b = reinterpret_cast<int32_t*>(take(8 * v->aln_cap));
  v->seq_rc = take(c.ld);
  return off;
}

// WorstCaseAlignmentScore (alignment_engine.cpp:101-110)
__host__ __device__ inline int64_t gap_score(const Scoring& s, int64_t len) {
  if (len == 0) return 0;
  int64_t a = s.g + (len - 1) * s.e, b = s.q + (len - 1) * s.c;
  return a < b ? a : b;
}
__host__ __device__ inline int64_t worst_case(const Scoring& s, int64_t i, int64_t j) {
  int64_t d = i > j ? i - j : j - i, mn = i < j ? i : j;
  int64_t a = -1 * (s.m * mn + gap_score(s, d));
  int64_t b = gap_score(s, i) + gap_score(s, j);
  return a < b ? a : b;
}
// Width rule (implementation.hpp:719-726): 16 int16 lanes or 8 int32 lanes
// per AVX2 vector, or 0 for "possible overflow".
__host__ __device__ inline int32_t lanes_for(const Scoring& s, uint32_t len, uint32_t nodes) {
  int64_t wc = worst_case(s, (int64_t)len + 8, nodes);
  if (wc < (int64_t)INT32_MIN + 1024) return 0;
  return wc < (int64_t)INT16_MIN + 1024 ? 8 : 16;
}

// Reverse complement of spoa's strand-ambiguous mode (biosoup 0.10.0
// Sequence::ReverseAndComplement: Watson-Crick / IUPAC pairing, reversed).
__host__ __device__ inline uint8_t complement_base(uint8_t ch) {
  switch (ch) {
    case 'A': return 'T';
    case 'C': return 'G';
    case 'G': return 'C';
    case 'T': return 'A';
    case 'U': return 'A';
    case 'R': return 'Y';
    case 'Y': return 'R';
    case 'K': return 'M';
    case 'M': return 'K';
    case 'B': return 'V';
    case 'D': return 'H';
    case 'H': return 'D';
    case 'V': return 'B';
    case 'a': return 't';
    case 'c': return 'g';
    case 'g': return 'c';
    case 't': return 'a';
    case 'u': return 'a';
    default: return ch;
  }
}

// Per-base weights of a read: explicit weights, Phred qualities (weight =
// quality - 33, graph.cpp:137-146; read back to front for a read kept on the
// reverse strand), or one constant weight (graph.cpp:119-125).
struct WeightSrc {
  const uint32_t* w;
  const uint8_t* qual;
  uint32_t len;
  uint32_t reversed;
  uint32_t wconst;
  __device__ __forceinline__ uint32_t at(uint32_t i) const {
    if (w) return w[i];
    if (qual) return (uint32_t)((int32_t)qual[reversed ? len - 1 - i : i] - 33);
    return wconst;
  }
};

// ---------------------------------------------------------------------------
// graph mutation (thread 0 of the CTA)
// ---------------------------------------------------------------------------
__device__ inline void g_reset(GraphView& G) {
  GraphHeader* h = G.hdr;
  h->n_nodes = h->n_edges = h->n_labels = h->n_seqs = h->num_codes = h->n_consensus = 0;
  h->status = kOk;
  for (int i = 0; i < 256; ++i) h->coder[i] = h->decoder[i] = -1;
}

// The graph's element counters, kept in registers while AddAlignment
// appends (thread 0 writes them back at the end): read back from the
// header after every append, they would make each step wait for the store
// of the step before.
struct GraphCounts {
  uint32_t nodes, edges, labels, seqs;
};
__device__ __forceinline__ GraphCounts g_counts(const GraphView& G) {
  const GraphHeader* h = G.hdr;
  return GraphCounts{h->n_nodes, h->n_edges, h->n_labels, h->n_seqs};
}
__device__ __forceinline__ void g_store_counts(GraphView& G, const GraphCounts& c) {
  GraphHeader* h = G.hdr;
  h->n_nodes = c.nodes;
  h->n_edges = c.edges;
  h->n_labels = c.labels;
  h->n_seqs = c.seqs;
}

__device__ inline int64_t g_add_node(GraphView& G, GraphCounts& c, uint32_t code) {
  if (c.nodes >= G.caps.nodes) return -1;
  uint32_t id = c.nodes++;
  G.code[id] = (uint8_t)code;
  G.nlink[id] = make_uint4(kNone, kNone, kNone, kNone);
  G.in_deg[id] = 0;
  G.n_aligned[id] = 0;
  G.nrec[id] = make_uint4(0, kNone, kNone, kNone);
  return id;
}
__device__ inline int64_t g_add_node(GraphView& G, uint32_t code) {
  GraphCounts c = g_counts(G);
  const int64_t id = g_add_node(G, c, code);
  g_store_counts(G, c);
  return id;
}

__device__ inline int g_add_label(GraphView& G, GraphCounts& c, uint32_t e) {
  if (c.labels >= G.caps.labels) return -1;
  uint32_t l = c.labels++;
  G.lab_seq[l] = c.seqs;
  G.lab_next[l] = kNone;
  const uint32_t last = G.e_lab_last[e];
  if (last != kNone) {
    G.lab_next[last] = l;
  } else {
    G.e_lab_first[e] = l;
  }
  G.e_lab_last[e] = l;
  return 0;
}

// A new edge tail -> head with weight w and no labels, appended to the
// tail's out-edge list and the head's in-edge list; -1 when full.
__device__ inline int64_t g_new_edge(GraphView& G, GraphCounts& c, uint32_t tail, uint32_t head,
                                     int64_t w) {
  if (c.edges >= G.caps.edges) return -1;
  uint32_t e = c.edges++;
  G.erec[e] = make_uint4(tail, head, kNone, kNone);
  G.e_weight[e] = w;
  G.e_lab_first[e] = G.e_lab_last[e] = kNone;
  const uint4 lt = G.nlink[tail];
  if (lt.w != kNone) G.erec[lt.w].w = e; else G.nlink[tail].z = e;
  G.nlink[tail].w = e;
  const uint4 lh = G.nlink[head];
  if (lh.y != kNone) G.erec[lh.y].z = e; else G.nlink[head].x = e;
  G.nlink[head].y = e;
  const uint32_t d = G.in_deg[head];
  G.in_deg[head] = d + 1;
  uint4 r = G.nrec[head];
  r.x = (r.x & 0xFFFF0000u) | min(d + 1, 0xFFFFu);
  if (d == 0) r.y = tail;
  if (d == 1) r.z = tail;
  if (d == 2) r.w = tail;
  G.nrec[head] = r;
  return e;
}
__device__ inline int64_t g_new_edge(GraphView& G, uint32_t tail, uint32_t head, int64_t w) {
  GraphCounts c = g_counts(G);
  const int64_t e = g_new_edge(G, c, tail, head, w);
  g_store_counts(G, c);
  return e;
}

// Graph::AddEdge (graph.cpp:81-91)
__device__ inline int g_add_edge(GraphView& G, GraphCounts& c, uint32_t tail, uint32_t head,
                                 uint32_t w) {
  for (uint32_t e = G.nlink[tail].z; e != kNone;) {
    const uint4 er = G.erec[e];
    if (er.y == head) {
      if (g_add_label(G, c, e)) return -1;
      G.e_weight[e] += w;
      return 0;
    }
    e = er.w;
  }
  const int64_t e = g_new_edge(G, c, tail, head, w);
  if (e < 0 || g_add_label(G, c, (uint32_t)e)) return -1;
  return 0;
}
__device__ inline int g_add_edge(GraphView& G, uint32_t tail, uint32_t head, uint32_t w) {
  GraphCounts c = g_counts(G);
  const int r = g_add_edge(G, c, tail, head, w);
  g_store_counts(G, c);
  return r;
}

// Graph::AddSequence (graph.cpp:93-110).  -1: empty range, -2: capacity.
__device__ inline int64_t g_add_sequence(GraphView& G, GraphCounts& c, const uint8_t* seq,
                                         const WeightSrc& w, uint32_t begin, uint32_t end) {
  if (begin == end) return -1;
  int64_t prev = -1;
  for (uint32_t i = begin; i < end; ++i) {
    int64_t curr = g_add_node(G, c, (uint32_t)G.hdr->coder[seq[i]]);
    if (curr < 0) return -2;
    if (prev >= 0) {
      // a new node has no out-edge yet: AddEdge always creates the edge
      const int64_t e = g_new_edge(G, c, (uint32_t)prev, (uint32_t)curr, w.at(i - 1) + w.at(i));
      if (e < 0 || g_add_label(G, c, (uint32_t)e)) return -2;
    }
    prev = curr;
  }
  return (int64_t)c.nodes - (end - begin);
}

// Graph::TopologicalSort (graph.cpp:249-303): the reference's iterative DFS
// over in-edges and aligned nodes, with its mark states (0 new, 1 in
// progress, 2 done) and ignored flags held as bitmaps in the graph arena.
// Every thread clears the bitmaps and prefetches the node records into L1,
// then thread 0 runs the DFS.  Returns 0, or -1 when the stack or the guard
// runs out (identical in every thread).
// The DFS of g_topo_sort_cta on one thread, the mark bitmaps already
// cleared: 0, or -1 when the stack or the guard runs out.
__device__ __forceinline__ int g_topo_dfs(GraphView& G) {
  const uint32_t nn = G.hdr->n_nodes;
  uint32_t* __restrict__ bits = G.sort_bits;
  auto bit = [&](uint32_t v, uint32_t kind) { return (bits[3 * (v >> 5) + kind] >> (v & 31)) & 1u; };
  auto set = [&](uint32_t v, uint32_t kind) { bits[3 * (v >> 5) + kind] |= 1u << (v & 31); };
  constexpr uint32_t kBusy = 0, kDone = 1, kIgn = 2;
  uint32_t* __restrict__ stack = G.stack;
  uint64_t sp = 0;
  auto push = [&](uint32_t v) -> bool {
    if (sp >= G.stack_cap) return false;
    stack[sp++] = v;
    return true;
  };
  uint32_t rank = 0;
  const uint32_t K = G.caps.aligned;
  // every iteration pops or pushes; pushes are bounded by the stack size
  uint64_t guard = 0;
  const uint64_t guard_max = 4 * G.stack_cap + 4 * (uint64_t)nn + 16;
  int rc = 0;
  for (uint32_t s = 0; s < nn && rc == 0; ++s) {
    if (bit(s, kDone) || bit(s, kBusy)) continue;
    push(s);
    while (sp) {
      if (++guard > guard_max) { rc = -1; break; }
      const uint32_t curr = stack[sp - 1];
      bool valid = true;
      if (!bit(curr, kDone)) {
        const uint4 r = G.nrec[curr];
        const uint32_t deg = r.x & 0xFFFFu, na = r.x >> 16;
        // in-edge tails in insertion order: three from the record, the
        // rest from the edge list
        if (deg > 0 && !bit(r.y, kDone)) { if (!push(r.y)) { rc = -1; break; } valid = false; }
        if (deg > 1 && !bit(r.z, kDone)) { if (!push(r.z)) { rc = -1; break; } valid = false; }
        if (deg > 2 && !bit(r.w, kDone)) { if (!push(r.w)) { rc = -1; break; } valid = false; }
        if (deg > 3) {
          uint32_t e = G.nlink[curr].x;
          for (int k = 0; k < 3 && e != kNone; ++k) e = G.erec[e].z;
          for (; e != kNone; e = G.erec[e].z) {
            const uint32_t tl = G.erec[e].x;
            if (!bit(tl, kDone)) { if (!push(tl)) { rc = -1; break; } valid = false; }
          }
          if (rc) break;
        }
        const uint32_t* al = G.aligned + (uint64_t)curr * K;
        const bool ign = bit(curr, kIgn);
        if (!ign) {
          for (uint32_t k = 0; k < na; ++k) {
            const uint32_t a = al[k];
            if (!bit(a, kDone)) {
              if (!push(a)) { rc = -1; break; }
              set(a, kIgn);
              valid = false;
            }
          }
          if (rc) break;
        }
        if (valid) {
          set(curr, kDone);
          if (!ign) {
            G.rank_to_node[rank] = curr;
            G.node_to_rank[curr] = rank++;
            for (uint32_t k = 0; k < na; ++k) {
              G.rank_to_node[rank] = al[k];
              G.node_to_rank[al[k]] = rank++;
            }
          }
        } else {
          set(curr, kBusy);
        }
      }
      if (valid) --sp;
    }
  }
  return (rc == 0 && rank == nn) ? 0 : -1;
}

static __device__ __noinline__ int g_topo_sort_cta(GraphView& G, int* s_ret) {
  const uint32_t nn = G.hdr->n_nodes;
  uint32_t* __restrict__ bits = G.sort_bits;
  const uint32_t words = 3 * ((nn + 31) / 32);
  for (uint32_t w = threadIdx.x; w < words; w += blockDim.x) bits[w] = 0;
#ifdef __CUDA_ARCH__
  for (uint32_t v = threadIdx.x * 8; v < nn; v += blockDim.x * 8)
    asm volatile("prefetch.global.L1 [%0];" ::"l"(G.nrec + v));
#endif
  __syncthreads();
  if (threadIdx.x == 0) *s_ret = g_topo_dfs(G);
  __syncthreads();
  return *s_ret;
}

__device__ inline int g_link_aligned(GraphView& G, uint32_t a, uint32_t b) {
  const uint32_t K = G.caps.aligned;
  if (G.n_aligned[a] >= K) return -1;
  G.aligned[(uint64_t)a * K + G.n_aligned[a]++] = b;
  G.nrec[a].x = (G.nrec[a].x & 0xFFFFu) | ((uint32_t)G.n_aligned[a] << 16);
  return 0;
}

// Read-only part of Graph::AddAlignment, run by every thread of the CTA
// before thread 0 adds (g_add_alignment with `pre`): for each aligned pair
// k (position not -1), pre[2k] = the existing node the reference reuses
// (the pair's node if its code matches, else an aligned node with the code)
// or kNone for a new node, and pre[2k+1] = the existing edge from the
// previous aligned pair's node to it, or kNone.  Exact because the read's
// path holds each node, and so each tail's out-edge list, at most once, and
// never two nodes of one aligned group: nothing the add changes is read
// here.  Characters new to the graph have no code yet (coder -1) and match
// no node.  Every thread must call it; ends with __syncthreads.
static __device__ __noinline__ void g_add_prepass(const GraphView& G, const int32_t* pairs,
                                                  uint32_t n_pairs, const uint8_t* seq,
                                                  uint32_t len, uint32_t* pre) {
  const GraphHeader* h = G.hdr;
  const uint32_t K = G.caps.aligned;
  for (uint32_t k = threadIdx.x; k < n_pairs; k += blockDim.x) {
    const int32_t nid = pairs[2 * k], pos = pairs[2 * k + 1];
    uint32_t node = kNone;
    if (pos >= 0 && (uint32_t)pos < len && nid >= 0 && (uint32_t)nid < h->n_nodes) {
      const uint32_t code = (uint32_t)h->coder[seq[pos]];
      if (G.code[nid] == code) {
        node = (uint32_t)nid;
      } else {
        const uint32_t na = G.n_aligned[nid];
        const uint32_t* al = G.aligned + (uint64_t)nid * K;
        for (uint32_t a = 0; a < na; ++a) {
          if (G.code[al[a]] == code) {
            node = al[a];
            break;
          }
        }
      }
    }
    pre[2 * k] = node;
  }
  __syncthreads();
  for (uint32_t k = threadIdx.x; k < n_pairs; k += blockDim.x) {
    uint32_t edge = kNone;
    const uint32_t head = pre[2 * k];
    if (pairs[2 * k + 1] != -1 && head != kNone) {
      // the previous aligned pair's node
      uint32_t tail = kNone;
      for (uint32_t b = k; b-- > 0;) {
        if (pairs[2 * b + 1] != -1) {
          tail = pre[2 * b];
          break;
        }
      }
      if (tail != kNone) {
        for (uint32_t e = G.nlink[tail].z; e != kNone; e = G.erec[e].w) {
          if (G.erec[e].y == head) {
            edge = e;
            break;
          }
        }
      }
    }
    pre[2 * k + 1] = edge;
  }
  __syncthreads();
}

// Graph::AddAlignment (graph.cpp:155-247) without its final
// TopologicalSort, which the caller runs with the whole CTA
// (g_topo_sort_cta).  pairs: n (node id | -1, position | -1).
static __device__ __noinline__ int32_t g_add_alignment(GraphView& G, const int32_t* pairs, uint32_t n_pairs,
                                          const uint8_t* seq, uint32_t len, const WeightSrc& w,
                                          const uint32_t* pre = nullptr) {
  GraphHeader* h = G.hdr;
  if (len == 0) return kOk;
  // room for the worst case of this read
  if ((uint64_t)h->n_nodes + len > G.caps.nodes || (uint64_t)h->n_edges + len + 1 > G.caps.edges ||
      (uint64_t)h->n_labels + len + 1 > G.caps.labels || h->n_seqs + 1 > G.caps.seqs)
    return kCapacity;
  for (uint32_t i = 0; i < len; ++i) {
    uint8_t ch = seq[i];
    if (h->coder[ch] == -1) {
      h->coder[ch] = (int32_t)h->num_codes;
      h->decoder[h->num_codes++] = ch;
    }
  }
  GraphCounts c = g_counts(G);
  // every exit leaves the counters in the header
  auto done = [&](int32_t st) {
    g_store_counts(G, c);
    return st;
  };
  if (n_pairs == 0) {
    int64_t b = g_add_sequence(G, c, seq, w, 0, len);
    if (b < -1) return done(kCapacity);
    G.seq_begin[c.seqs++] = (uint32_t)b;
    return done(kOk);  // the caller re-sorts (g_topo_sort_cta)
  }
  int32_t first_valid = -1, last_valid = -1;
  for (uint32_t k = 0; k < n_pairs; ++k) {
    int32_t pos = pairs[2 * k + 1];
    if (pos != -1) {
      if (pos < 0 || pos >= (int32_t)len) return kInvalidAlignment;
      if (first_valid == -1) first_valid = pos;
      last_valid = pos;
    }
  }
  if (first_valid == -1) return kMissingSequence;
  for (uint32_t k = 0; k < n_pairs; ++k) {
    int32_t nid = pairs[2 * k];
    if (nid < -1 || nid >= (int32_t)c.nodes) return kInvalidAlignment;
  }
  int64_t begin = g_add_sequence(G, c, seq, w, 0, (uint32_t)first_valid);
  if (begin < -1) return done(kCapacity);
  int64_t prev = begin >= 0 ? (int64_t)c.nodes - 1 : -1;
  int64_t last = g_add_sequence(G, c, seq, w, (uint32_t)last_valid + 1, len);
  if (last < -1) return done(kCapacity);
  const uint32_t K = G.caps.aligned;
  bool prev_new = true;  // prev was created by this read (it has no edge to an old node)
  for (uint32_t k = 0; k < n_pairs; ++k) {
    int32_t nid = pairs[2 * k], pos = pairs[2 * k + 1];
    if (pos == -1) continue;
    uint32_t code = (uint32_t)h->coder[seq[pos]];
    int64_t curr = -1;
    bool curr_new = false;
    if (pre) {
      if (pre[2 * k] != kNone) curr = pre[2 * k];
    } else if (nid != -1) {
      if (G.code[nid] == code) {
        curr = nid;
      } else {
        const uint32_t na = G.n_aligned[nid];
        const uint32_t* al = G.aligned + (uint64_t)nid * K;
        for (uint32_t a = 0; a < na; ++a) {
          if (G.code[al[a]] == code) {
            curr = al[a];
            break;
          }
        }
      }
    }
    if (curr < 0) {
      curr = g_add_node(G, c, code);
      if (curr < 0) return done(kCapacity);
      curr_new = true;
      if (nid != -1) {
        const uint32_t na = G.n_aligned[nid];
        const uint32_t* al = G.aligned + (uint64_t)nid * K;
        for (uint32_t a = 0; a < na; ++a) {
          uint32_t kt = al[a];
          if (g_link_aligned(G, kt, (uint32_t)curr) || g_link_aligned(G, (uint32_t)curr, kt))
            return done(kCapacity);
        }
        if (g_link_aligned(G, (uint32_t)nid, (uint32_t)curr) ||
            g_link_aligned(G, (uint32_t)curr, (uint32_t)nid))
          return done(kCapacity);
      }
    }
    if (begin < 0) begin = curr;
    if (prev >= 0) {
      const uint32_t wt = w.at(pos - 1) + w.at(pos);
      if (!pre) {
        if (g_add_edge(G, c, (uint32_t)prev, (uint32_t)curr, wt)) return done(kCapacity);
      } else if (!prev_new && !curr_new && pre[2 * k + 1] != kNone) {
        // AddEdge on an existing edge: one more label and the weight
        const uint32_t e = pre[2 * k + 1];
        if (g_add_label(G, c, e)) return done(kCapacity);
        G.e_weight[e] += wt;
      } else {
        const int64_t e = g_new_edge(G, c, (uint32_t)prev, (uint32_t)curr, wt);
        if (e < 0 || g_add_label(G, c, (uint32_t)e)) return done(kCapacity);
      }
    }
    prev = curr;
    prev_new = curr_new;
  }
  if (last >= 0) {
    if (g_add_edge(G, c, (uint32_t)prev, (uint32_t)last, w.at(last_valid) + w.at(last_valid + 1)))
      return done(kCapacity);
  }
  G.seq_begin[c.seqs++] = (uint32_t)begin;
  return done(kOk);  // the caller re-sorts (g_topo_sort_cta)
}

// ---------------------------------------------------------------------------
// consensus (graph.cpp:433-516), thread 0
// ---------------------------------------------------------------------------
__device__ inline uint32_t g_branch_completion(GraphView& G, uint32_t rank) {
  const uint32_t start = G.rank_to_node[rank];
  for (uint32_t e = G.nlink[start].z; e != kNone; e = G.erec[e].w) {
    uint32_t hd = G.erec[e].y;
    for (uint32_t f = G.nlink[hd].x; f != kNone; f = G.erec[f].z) {
      uint32_t t = G.erec[f].x;
      if (t != start) G.cscore[t] = -1;
    }
  }
  uint32_t mx = kNone;
  const uint32_t nn = G.hdr->n_nodes;
  for (uint32_t r = rank + 1; r < nn; ++r) {
    uint32_t it = G.rank_to_node[r];
    G.cscore[it] = -1;
    G.cpred[it] = kNone;
    for (uint32_t f = G.nlink[it].x; f != kNone; f = G.erec[f].z) {
      uint32_t t = G.erec[f].x;
      if (G.cscore[t] == -1) continue;
      int64_t w = G.e_weight[f];
      if (G.cscore[it] < w || (G.cscore[it] == w && G.cscore[G.cpred[it]] <= G.cscore[t])) {
        G.cscore[it] = w;
        G.cpred[it] = t;
      }
    }
    if (G.cpred[it] != kNone) G.cscore[it] += G.cscore[G.cpred[it]];
    if (mx == kNone || G.cscore[mx] < G.cscore[it]) mx = it;
  }
  return mx;
}

static __device__ __noinline__ void g_consensus(GraphView& G) {
  const uint32_t nn = G.hdr->n_nodes;
  G.hdr->n_consensus = 0;
  if (nn == 0) return;
  for (uint32_t i = 0; i < nn; ++i) {
    G.cscore[i] = -1;
    G.cpred[i] = kNone;
  }
  uint32_t mx = kNone;
  for (uint32_t r = 0; r < nn; ++r) {
    uint32_t it = G.rank_to_node[r];
    for (uint32_t f = G.nlink[it].x; f != kNone; f = G.erec[f].z) {
      uint32_t t = G.erec[f].x;
      int64_t w = G.e_weight[f];
      if (G.cscore[it] < w || (G.cscore[it] == w && G.cscore[G.cpred[it]] <= G.cscore[t])) {
        G.cscore[it] = w;
        G.cpred[it] = t;
      }
    }
    if (G.cpred[it] != kNone) G.cscore[it] += G.cscore[G.cpred[it]];
    if (mx == kNone || G.cscore[mx] < G.cscore[it]) mx = it;
  }
  // each completion moves to a strictly later rank
  while (G.nlink[mx].z != kNone) {
    uint32_t nx = g_branch_completion(G, G.node_to_rank[mx]);
    if (nx == kNone) break;
    mx = nx;
  }
  uint32_t n = 0;
  while (G.cpred[mx] != kNone && n < nn) {
    G.consensus[n++] = mx;
    mx = G.cpred[mx];
  }
  G.consensus[n++] = mx;
  for (uint32_t a = 0, b = n - 1; a < b; ++a, --b) {
    uint32_t t = G.consensus[a];
    G.consensus[a] = G.consensus[b];
    G.consensus[b] = t;
  }
  G.hdr->n_consensus = n;
}

// Node::Successor (graph.cpp:22-30)
__device__ inline uint32_t g_successor(const GraphView& G, uint32_t node, uint32_t label) {
  for (uint32_t e = G.nlink[node].z; e != kNone; e = G.erec[e].w) {
    for (uint32_t l = G.e_lab_first[e]; l != kNone; l = G.lab_next[l]) {
      if (G.lab_seq[l] == label) return G.erec[e].y;
      if (G.lab_seq[l] > label) break;  // labels are appended in sequence order
    }
  }
  return kNone;
}

// InitializeMultipleSequenceAlignment (graph.cpp:321-337); returns row size.
__device__ inline uint32_t g_msa_columns(GraphView& G) {
  const uint32_t nn = G.hdr->n_nodes, K = G.caps.aligned;
  uint32_t j = 0;
  for (uint32_t i = 0; i < nn; ++i, ++j) {
    uint32_t it = G.rank_to_node[i];
    G.column[it] = j;
    const uint32_t na = G.n_aligned[it];
    for (uint32_t k = 0; k < na; ++k) {
      G.column[G.aligned[(uint64_t)it * K + k]] = j;
      ++i;
    }
  }
  return j;
}


// ---------------------------------------------------------------------------
// Graph::Subgraph and graph loading (thread 0)
// ---------------------------------------------------------------------------
// Graph::Subgraph (graph.cpp:541-595) of S into the empty graph D, without
// the final sort.  The node set is ExtractSubgraph's (graph.cpp:518-539):
// every node reachable from `end` over in-edges and aligned nodes, not
// expanded below id `begin`; it is a set, so the stack may visit it in any
// order.  Its nodes are added in id order (map[k] = id in S of node k of
// D), then, node by node, each in-edge whose tail is in the set with the
// edge's weight (one label, sequence 0, as AddEdge gives it on a graph
// without sequences) and the aligned nodes in the set, in list order.
// gid (one word per node of S) must hold kNone on entry; stack is scratch.
// Returns kOk, or kCapacity when D or the stack is too small.
__device__ inline int32_t g_subgraph_build(const GraphView& S, GraphView& D, uint32_t begin,
                                           uint32_t end, uint32_t* gid, uint32_t* stack,
                                           uint64_t stack_cap, uint32_t* map) {
  const uint32_t nn = S.hdr->n_nodes;
  constexpr uint32_t kIn = 0xFFFFFFFEu;  // in the set, not numbered yet
  int32_t st = kOk;
  g_reset(D);
  D.hdr->num_codes = S.hdr->num_codes;
  for (int k = 0; k < 256; ++k) {
    D.hdr->coder[k] = S.hdr->coder[k];
    D.hdr->decoder[k] = S.hdr->decoder[k];
  }
  const uint32_t KS = S.caps.aligned;
  uint64_t sp = 0;
  if (end < nn) stack[sp++] = end;
  while (sp && st == kOk) {
    const uint32_t v = stack[--sp];
    if (gid[v] != kNone || v < begin) continue;
    gid[v] = kIn;
    for (uint32_t e = S.nlink[v].x; e != kNone; e = S.erec[e].z) {
      if (sp >= stack_cap) { st = kCapacity; break; }
      stack[sp++] = S.erec[e].x;
    }
    for (uint32_t k = 0; k < S.n_aligned[v] && st == kOk; ++k) {
      if (sp >= stack_cap) { st = kCapacity; break; }
      stack[sp++] = S.aligned[(uint64_t)v * KS + k];
    }
  }
  for (uint32_t v = 0; v < nn && st == kOk; ++v) {
    if (gid[v] != kIn) continue;
    const int64_t id = g_add_node(D, S.code[v]);
    if (id < 0) { st = kCapacity; break; }
    gid[v] = (uint32_t)id;
    map[id] = v;
  }
  for (uint32_t v = 0; v < nn && st == kOk; ++v) {
    const uint32_t h = gid[v];
    if (h == kNone) continue;
    for (uint32_t e = S.nlink[v].x; e != kNone; e = S.erec[e].z) {
      const uint32_t t = gid[S.erec[e].x];
      // AddEdge takes a 32-bit weight (graph.cpp:81)
      if (t != kNone && g_add_edge(D, t, h, (uint32_t)S.e_weight[e])) { st = kCapacity; break; }
    }
    for (uint32_t k = 0; k < S.n_aligned[v] && st == kOk; ++k) {
      const uint32_t a = gid[S.aligned[(uint64_t)v * KS + k]];
      if (a != kNone && g_link_aligned(D, h, a)) st = kCapacity;
    }
  }
  return st;
}

// A saved graph (arrays checked by the caller: every id in range, one rank
// per node, at most caps.aligned aligned nodes per node).
struct ImportArgs {
  uint32_t n_nodes, n_edges, n_seqs, n_pairs, n_consensus, num_codes;
  const uint8_t* codes;
  const uint32_t *e_tail, *e_head;
  const int64_t* e_weight;
  const uint32_t *lab_off, *labels;  // labels of edge e: lab_off[e] .. lab_off[e + 1]
  const uint32_t *seq_begin, *pairs, *rank, *consensus;
  const int32_t *coder, *decoder;
};

// Rebuilds a saved graph in the empty graph G the way the reference's
// Graph::load (include/spoa/graph.hpp:236-275) rebuilds it: nodes in id
// order; edges in id order, each appended to its tail's out-edge list and
// its head's in-edge list, with its labels and weight; for every aligned
// pair (a, b) in order, b appended to a's list and a to b's (which can
// reorder a node's aligned list against the saved graph, as the
// reference's load does); rank order, sequence starts and the last
// consensus as saved.  Returns kOk or kCapacity.
__device__ inline int32_t g_import(GraphView& G, const ImportArgs& a) {
  int32_t st = kOk;
  GraphHeader* h = G.hdr;
  g_reset(G);
  h->num_codes = a.num_codes;
  for (int k = 0; k < 256; ++k) {
    h->coder[k] = a.coder[k];
    h->decoder[k] = a.decoder[k];
  }
  for (uint32_t v = 0; v < a.n_nodes && st == kOk; ++v)
    if (g_add_node(G, a.codes[v]) < 0) st = kCapacity;
  for (uint32_t e = 0; e < a.n_edges && st == kOk; ++e) {
    const int64_t id = g_new_edge(G, a.e_tail[e], a.e_head[e], a.e_weight[e]);
    if (id < 0) {
      st = kCapacity;
      break;
    }
    for (uint32_t k = a.lab_off[e]; k < a.lab_off[e + 1]; ++k) {
      if (h->n_labels >= G.caps.labels) {
        st = kCapacity;
        break;
      }
      const uint32_t l = h->n_labels++;
      G.lab_seq[l] = a.labels[k];
      G.lab_next[l] = kNone;
      if (G.e_lab_last[id] != kNone) G.lab_next[G.e_lab_last[id]] = l; else G.e_lab_first[id] = l;
      G.e_lab_last[id] = l;
    }
  }
  for (uint32_t k = 0; k < a.n_pairs && st == kOk; ++k) {
    const uint32_t x = a.pairs[2 * k], y = a.pairs[2 * k + 1];
    if (g_link_aligned(G, x, y) || g_link_aligned(G, y, x)) st = kCapacity;
  }
  if (st == kOk) {
    for (uint32_t r = 0; r < a.n_nodes; ++r) {
      G.rank_to_node[r] = a.rank[r];
      G.node_to_rank[a.rank[r]] = r;
    }
    for (uint32_t s = 0; s < a.n_seqs; ++s) G.seq_begin[s] = a.seq_begin[s];
    h->n_seqs = a.n_seqs;
    for (uint32_t k = 0; k < a.n_consensus; ++k) G.consensus[k] = a.consensus[k];
    h->n_consensus = a.n_consensus;
  }
  return st;
}

}  // namespace spoa_gb300
