// device_graph_host.cpp - the device graph code of spoa_gb300/csrc/
// poa_device.cuh (AddAlignment, the topological sort, consensus, subgraph
// extraction, graph loading) compiled for the host, single-threaded, so the
// CPU test suite can compare it with the oracle step by step
// (tests/test_device_graph_host.py).  TEST INFRASTRUCTURE ONLY: the product
// runs the same functions on the GPU.
//
// The CUDA qualifiers become nothing, the CTA is one thread (threadIdx.x 0,
// blockDim.x 1, __syncthreads a no-op), and uint4 is a plain struct.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#define __host__
#define __device__
#define __forceinline__ inline
#define __noinline__
struct uint4 {
  unsigned int x, y, z, w;
};
static inline uint4 make_uint4(unsigned a, unsigned b, unsigned c, unsigned d) {
  return uint4{a, b, c, d};
}
using std::max;
using std::min;
struct HostDim {
  unsigned x;
};
static const HostDim threadIdx{0}, blockDim{1};
static inline void __syncthreads() {}

#include "../../spoa_gb300/csrc/poa_device.cuh"

using namespace spoa_gb300;

struct DG {
  std::vector<uint8_t> buf;
  GraphView v;
};

extern "C" {

DG* dg_create(uint32_t nodes, uint32_t edges, uint32_t labels, uint32_t seqs, uint32_t aligned) {
  DG* g = new DG();
  GraphCaps c{nodes, edges, labels, seqs, aligned};
  g->buf.resize(graph_layout(nullptr, c, &g->v) + 256);
  graph_layout(g->buf.data(), c, &g->v);
  g_reset(g->v);
  return g;
}

void dg_destroy(DG* g) { delete g; }

// Graph::AddAlignment, then the sort (graph.cpp:155-303); with_prepass runs
// the read-only pre-pass first and lets the add use its results
int32_t dg_add(DG* g, const int32_t* pairs, uint32_t n_pairs, const char* seq, uint32_t len,
               const uint32_t* weights, int32_t with_prepass) {
  WeightSrc ws{weights, nullptr, len, 0u, 1u};
  const uint8_t* s = reinterpret_cast<const uint8_t*>(seq);
  std::vector<uint32_t> pre(2 * (size_t)n_pairs + 2);
  if (with_prepass) g_add_prepass(g->v, pairs, n_pairs, s, len, pre.data());
  int32_t st = g_add_alignment(g->v, pairs, n_pairs, s, len, ws, with_prepass ? pre.data() : nullptr);
  if (st != kOk) return st;
  int ret = 0;
  if (len > 0 && g_topo_sort_cta(g->v, &ret) != 0) return kCapacity;
  return kOk;
}

// nodes, edges, sequences, consensus, labels, num_codes
void dg_counts(const DG* g, uint32_t* out) {
  const GraphHeader* h = g->v.hdr;
  out[0] = h->n_nodes;
  out[1] = h->n_edges;
  out[2] = h->n_seqs;
  out[3] = h->n_consensus;
  out[4] = h->n_labels;
  out[5] = h->num_codes;
}

// node characters, rank order, edges by id (tail, head, weight, label CSR),
// aligned lists (CSR), sequence starts, consensus node ids
void dg_export(const DG* g, uint8_t* chars, uint32_t* rank, uint32_t* e_tail, uint32_t* e_head,
               int64_t* e_weight, uint32_t* lab_off, uint32_t* labels, uint32_t* al_off,
               uint32_t* al, uint32_t* seq_begin, uint32_t* consensus) {
  const GraphView& G = g->v;
  const GraphHeader* h = G.hdr;
  uint32_t na = 0;
  for (uint32_t v = 0; v < h->n_nodes; ++v) {
    chars[v] = (uint8_t)h->decoder[G.code[v]];
    rank[v] = G.rank_to_node[v];
    al_off[v] = na;
    for (uint32_t k = 0; k < G.n_aligned[v]; ++k) al[na++] = G.aligned[(uint64_t)v * G.caps.aligned + k];
  }
  al_off[h->n_nodes] = na;
  uint32_t nl = 0;
  for (uint32_t e = 0; e < h->n_edges; ++e) {
    e_tail[e] = G.erec[e].x;
    e_head[e] = G.erec[e].y;
    e_weight[e] = G.e_weight[e];
    lab_off[e] = nl;
    for (uint32_t l = G.e_lab_first[e]; l != kNone; l = G.lab_next[l]) labels[nl++] = G.lab_seq[l];
  }
  lab_off[h->n_edges] = nl;
  for (uint32_t s = 0; s < h->n_seqs; ++s) seq_begin[s] = G.seq_begin[s];
  for (uint32_t k = 0; k < h->n_consensus; ++k) consensus[k] = G.consensus[k];
}

// Graph::GenerateConsensus (graph.cpp:368-375); returns the length
uint32_t dg_consensus(DG* g, char* out, uint32_t cap) {
  g_consensus(g->v);
  const GraphHeader* h = g->v.hdr;
  for (uint32_t k = 0; k < h->n_consensus && k < cap; ++k)
    out[k] = (char)h->decoder[g->v.code[g->v.consensus[k]]];
  return h->n_consensus;
}

// Graph::Subgraph (graph.cpp:541-595) into dst, sorted; map gets the source
// id of each subgraph node
int32_t dg_subgraph(const DG* src, uint32_t begin, uint32_t end, DG* dst, uint32_t* map) {
  const uint32_t nn = src->v.hdr->n_nodes;
  std::vector<uint32_t> gid(nn + 1, kNone);
  const uint64_t cap = (uint64_t)src->v.hdr->n_edges + (uint64_t)nn * src->v.caps.aligned + 1;
  std::vector<uint32_t> stack(cap);
  int32_t st = g_subgraph_build(src->v, dst->v, begin, end, gid.data(), stack.data(), cap, map);
  if (st != kOk) return st;
  int ret = 0;
  return g_topo_sort_cta(dst->v, &ret) != 0 ? kCapacity : kOk;
}

// save then load: the fields the reference's Graph::save archives, in its
// order (aligned pairs a < b, node order then list order), rebuilt in dst
int32_t dg_reload(const DG* src, DG* dst) {
  const GraphView& S = src->v;
  const GraphHeader* h = S.hdr;
  const uint32_t N = h->n_nodes, E = h->n_edges;
  std::vector<uint8_t> codes(N + 1);
  std::vector<uint32_t> tail(E + 1), head(E + 1), lab_off(E + 1), labels, pairs, rank(N + 1),
      sb(h->n_seqs + 1), cons(h->n_consensus + 1);
  std::vector<int64_t> weight(E + 1);
  for (uint32_t v = 0; v < N; ++v) {
    codes[v] = S.code[v];
    rank[v] = S.rank_to_node[v];
    for (uint32_t k = 0; k < S.n_aligned[v]; ++k) {
      const uint32_t b = S.aligned[(uint64_t)v * S.caps.aligned + k];
      if (v < b) {
        pairs.push_back(v);
        pairs.push_back(b);
      }
    }
  }
  for (uint32_t e = 0; e < E; ++e) {
    tail[e] = S.erec[e].x;
    head[e] = S.erec[e].y;
    weight[e] = S.e_weight[e];
    lab_off[e] = (uint32_t)labels.size();
    for (uint32_t l = S.e_lab_first[e]; l != kNone; l = S.lab_next[l]) labels.push_back(S.lab_seq[l]);
  }
  lab_off[E] = (uint32_t)labels.size();
  labels.push_back(0);
  pairs.push_back(0);
  for (uint32_t s = 0; s < h->n_seqs; ++s) sb[s] = S.seq_begin[s];
  for (uint32_t k = 0; k < h->n_consensus; ++k) cons[k] = S.consensus[k];
  ImportArgs a;
  a.n_nodes = N;
  a.n_edges = E;
  a.n_seqs = h->n_seqs;
  a.n_pairs = (uint32_t)(pairs.size() - 1) / 2;
  a.n_consensus = h->n_consensus;
  a.num_codes = h->num_codes;
  a.codes = codes.data();
  a.e_tail = tail.data();
  a.e_head = head.data();
  a.e_weight = weight.data();
  a.lab_off = lab_off.data();
  a.labels = labels.data();
  a.seq_begin = sb.data();
  a.pairs = pairs.data();
  a.rank = rank.data();
  a.consensus = cons.data();
  a.coder = h->coder;
  a.decoder = h->decoder;
  return g_import(dst->v, a);
}

}  // extern "C"
