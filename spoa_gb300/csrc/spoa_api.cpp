// spoa_api.cpp - spoa's C++ API (include/spoa/*.hpp) over the C ABI of
// libspoa_gb300.so.  Host code only: every DP, graph update, consensus and
// MSA runs on the GPU; this layer converts types, maps status codes to
// spoa's std::invalid_argument messages and rebuilds the host views of the
// graph from a device export.
#include <algorithm>
#include <cstring>
#include <fstream>
#include <stdexcept>
#include <string>
#include <unordered_set>
#include <utility>
#include <vector>

#include "spoa/spoa.hpp"
#include "spoa_gb300.h"

namespace spoa {

namespace {

// "[spoa::<where>] error: <message>" as the reference throws it.
[[noreturn]] void Throw(const std::string& where, const std::string& message) {
  throw std::invalid_argument("[spoa::" + where + "] error: " + message);
}

void Check(const std::string& where, int32_t status) {
  if (status == SPOA_GB300_OK) return;
  Throw(where, spoa_gb300_status_string(status));
}

std::vector<int32_t> FlattenAlignment(const Alignment& alignment) {
  std::vector<int32_t> pairs(2 * alignment.size());
  for (std::size_t k = 0; k < alignment.size(); ++k) {
    pairs[2 * k] = alignment[k].first;
    pairs[2 * k + 1] = alignment[k].second;
  }
  return pairs;
}

// The engine of this library: one device DP arena, grown on demand.
class CudaAlignmentEngine : public AlignmentEngine {
 public:
  CudaAlignmentEngine(spoa_gb300_engine* handle, AlignmentType type, AlignmentSubtype subtype,
                      const int8_t* p)
      : AlignmentEngine(type, subtype, p[0], p[1], p[2], p[3], p[4], p[5]), handle_(handle) {}

  ~CudaAlignmentEngine() override { spoa_gb300_engine_destroy(handle_); }

  CudaAlignmentEngine(const CudaAlignmentEngine&) = delete;
  CudaAlignmentEngine& operator=(const CudaAlignmentEngine&) = delete;

  // simd_alignment_engine_implementation.hpp:381-422
  void Prealloc(std::uint32_t max_sequence_len, std::uint8_t alphabet_size) override {
    Check("CudaAlignmentEngine::Prealloc",
          spoa_gb300_engine_prealloc(handle_, max_sequence_len, alphabet_size));
  }

  // simd_alignment_engine_implementation.hpp:703-780
  Alignment Align(const char* sequence, std::uint32_t sequence_len, const Graph& graph,
                  std::int32_t* score) override {
    uint32_t n_nodes = 0, ne = 0, ns = 0, nc = 0, nl = 0, codes = 0;
    Check("CudaAlignmentEngine::Align",
          spoa_gb300_graph_counts(graph.device(), &n_nodes, &ne, &ns, &nc, &nl, &codes));
    std::vector<int32_t> pairs(2 * (static_cast<std::size_t>(n_nodes) + sequence_len + 16));
    int32_t s = 0, written = 0;
    uint32_t n_pairs = 0;
    Check("CudaAlignmentEngine::Align",
          spoa_gb300_engine_align(handle_, sequence, sequence_len, graph.device(), &s, &written,
                                  pairs.data(), static_cast<uint32_t>(pairs.size() / 2),
                                  &n_pairs));
    if (written && score) *score = s;
    Alignment alignment(n_pairs);
    for (uint32_t k = 0; k < n_pairs; ++k) alignment[k] = {pairs[2 * k], pairs[2 * k + 1]};
    return alignment;
  }

 private:
  spoa_gb300_engine* handle_;
};

}  // namespace

// ---------------------------------------------------------------------------
// AlignmentEngine (alignment_engine.cpp of the reference)
// ---------------------------------------------------------------------------

AlignmentEngine::AlignmentEngine(AlignmentType type, AlignmentSubtype subtype, std::int8_t m,
                                 std::int8_t n, std::int8_t g, std::int8_t e, std::int8_t q,
                                 std::int8_t c)
    : type_(type), subtype_(subtype), m_(m), n_(n), g_(g), e_(e), q_(q), c_(c) {}

std::unique_ptr<AlignmentEngine> AlignmentEngine::Create(AlignmentType type, std::int8_t m,
                                                         std::int8_t n, std::int8_t g) {
  return Create(type, m, n, g, g);
}

std::unique_ptr<AlignmentEngine> AlignmentEngine::Create(AlignmentType type, std::int8_t m,
                                                         std::int8_t n, std::int8_t g,
                                                         std::int8_t e) {
  return Create(type, m, n, g, e, g, e);
}

std::unique_ptr<AlignmentEngine> AlignmentEngine::Create(AlignmentType type, std::int8_t m,
                                                         std::int8_t n, std::int8_t g,
                                                         std::int8_t e, std::int8_t q,
                                                         std::int8_t c) {
  const int32_t t = static_cast<int32_t>(type);
  if (t < 0 || t > 2) Throw("AlignmentEngine::Create", "invalid alignment type!");
  if (g > 0 || q > 0) Throw("AlignmentEngine::Create", "gap opening penalty must be non-positive!");
  if (e > 0 || c > 0) Throw("AlignmentEngine::Create", "gap extension penalty must be non-positive!");
  spoa_gb300_engine* h = nullptr;
  Check("AlignmentEngine::Create", spoa_gb300_engine_create(t, m, n, g, e, q, c, &h));
  int32_t rtype = 0, rsub = 0;
  int8_t p[6];
  const int32_t st = spoa_gb300_engine_params(h, &rtype, &rsub, p);
  if (st != SPOA_GB300_OK) {
    spoa_gb300_engine_destroy(h);
    Check("AlignmentEngine::Create", st);
  }
  return std::unique_ptr<AlignmentEngine>(new CudaAlignmentEngine(
      h, static_cast<AlignmentType>(rtype), static_cast<AlignmentSubtype>(rsub), p));
}

Alignment AlignmentEngine::Align(const std::string& sequence, const Graph& graph,
                                 std::int32_t* score) {
  return Align(sequence.c_str(), static_cast<std::uint32_t>(sequence.size()), graph, score);
}

std::int64_t AlignmentEngine::WorstCaseAlignmentScore(std::int64_t i, std::int64_t j) const {
  auto gap = [&](std::int64_t len) -> std::int64_t {
    if (len == 0) return 0;
    return std::min<std::int64_t>(g_ + (len - 1) * e_, q_ + (len - 1) * c_);
  };
  return std::min(-1 * (m_ * std::min(i, j) + gap(i < j ? j - i : i - j)), gap(i) + gap(j));
}

// ---------------------------------------------------------------------------
// Graph::Node / Graph::Edge (graph.cpp:12-63)
// ---------------------------------------------------------------------------

Graph::Node::Node(std::uint32_t id, std::uint32_t code) : id(id), code(code) {}

Graph::Node* Graph::Node::Successor(std::uint32_t label) const {
  for (const Edge* e : outedges)
    if (std::find(e->labels.begin(), e->labels.end(), label) != e->labels.end()) return e->head;
  return nullptr;
}

std::uint32_t Graph::Node::Coverage() const {
  std::unordered_set<std::uint32_t> seen;
  for (const Edge* e : inedges) seen.insert(e->labels.begin(), e->labels.end());
  for (const Edge* e : outedges) seen.insert(e->labels.begin(), e->labels.end());
  return static_cast<std::uint32_t>(seen.size());
}

Graph::Edge::Edge(Node* tail, Node* head, std::uint32_t label, std::uint32_t weight)
    : tail(tail), head(head), labels(1, label), weight(weight) {}

void Graph::Edge::AddSequence(std::uint32_t label, std::uint32_t w) {
  labels.push_back(label);
  weight += w;
}

// ---------------------------------------------------------------------------
// Graph
// ---------------------------------------------------------------------------

Graph::Graph() : handle_(nullptr), view_valid_(false), num_codes_(0) {
  Check("Graph::Graph", spoa_gb300_graph_create(&handle_));
}

Graph::Graph(Graph&& o) noexcept
    : handle_(o.handle_),
      view_valid_(o.view_valid_),
      num_codes_(o.num_codes_),
      coder_(std::move(o.coder_)),
      decoder_(std::move(o.decoder_)),
      nodes_(std::move(o.nodes_)),
      edges_(std::move(o.edges_)),
      rank_to_node_(std::move(o.rank_to_node_)),
      sequences_(std::move(o.sequences_)),
      consensus_(std::move(o.consensus_)) {
  o.handle_ = nullptr;
  o.view_valid_ = false;
}

Graph& Graph::operator=(Graph&& o) noexcept {
  if (this != &o) {
    if (handle_) spoa_gb300_graph_destroy(handle_);
    handle_ = o.handle_;
    view_valid_ = o.view_valid_;
    num_codes_ = o.num_codes_;
    coder_ = std::move(o.coder_);
    decoder_ = std::move(o.decoder_);
    nodes_ = std::move(o.nodes_);
    edges_ = std::move(o.edges_);
    rank_to_node_ = std::move(o.rank_to_node_);
    sequences_ = std::move(o.sequences_);
    consensus_ = std::move(o.consensus_);
    o.handle_ = nullptr;
    o.view_valid_ = false;
  }
  return *this;
}

Graph::~Graph() {
  if (handle_) spoa_gb300_graph_destroy(handle_);
}

void Graph::Refresh() const {
  if (view_valid_) return;
  uint32_t N = 0, E = 0, S = 0, Cn = 0, Lb = 0, codes = 0;
  Check("Graph::Graph", spoa_gb300_graph_counts(handle_, &N, &E, &S, &Cn, &Lb, &codes));
  auto sz = [](uint32_t k) { return std::max<std::size_t>(k, 1); };
  std::vector<uint8_t> chars(sz(N)), code(sz(N));
  std::vector<uint32_t> in_off(N + 1), in_e(sz(E)), out_off(N + 1), out_e(sz(E));
  std::vector<uint32_t> al_off(N + 1), al(sz(N) * 64);
  std::vector<uint32_t> et(sz(E)), eh(sz(E)), lab_off(E + 1), labs(sz(Lb));
  std::vector<int64_t> ew(sz(E));
  std::vector<uint32_t> rank(sz(N)), sb(sz(S)), cons(sz(Cn));
  coder_.assign(256, -1);
  decoder_.assign(256, -1);
  Check("Graph::Graph",
        spoa_gb300_graph_export(handle_, chars.data(), code.data(), in_off.data(), in_e.data(),
                                out_off.data(), out_e.data(), al_off.data(), al.data(),
                                et.data(), eh.data(), ew.data(), lab_off.data(), labs.data(),
                                rank.data(), sb.data(), cons.data(), coder_.data(),
                                decoder_.data()));
  num_codes_ = codes;
  // Nodes and edges are only appended until Clear: the objects of the last
  // view are updated in place and new ones appended, so pointers to them
  // survive the refresh.
  if (nodes_.size() > N) nodes_.resize(N);
  if (edges_.size() > E) edges_.resize(E);
  nodes_.reserve(N);
  edges_.reserve(E);
  for (uint32_t v = 0; v < N; ++v) {
    if (v < nodes_.size()) {
      Node* node = nodes_[v].get();
      node->code = code[v];
      node->inedges.clear();
      node->outedges.clear();
      node->aligned_nodes.clear();
    } else {
      nodes_.emplace_back(new Node(v, code[v]));
    }
  }
  for (uint32_t k = 0; k < E; ++k) {
    if (k >= edges_.size()) edges_.emplace_back(new Edge(nullptr, nullptr, 0, 0));
    Edge* ed = edges_[k].get();
    ed->tail = nodes_[et[k]].get();
    ed->head = nodes_[eh[k]].get();
    ed->labels.assign(labs.begin() + lab_off[k], labs.begin() + lab_off[k + 1]);
    ed->weight = ew[k];
  }
  for (uint32_t v = 0; v < N; ++v) {
    Node* node = nodes_[v].get();
    for (uint32_t k = in_off[v]; k < in_off[v + 1]; ++k) node->inedges.push_back(edges_[in_e[k]].get());
    for (uint32_t k = out_off[v]; k < out_off[v + 1]; ++k)
      node->outedges.push_back(edges_[out_e[k]].get());
    for (uint32_t k = al_off[v]; k < al_off[v + 1]; ++k)
      node->aligned_nodes.push_back(nodes_[al[k]].get());
  }
  rank_to_node_.clear();
  for (uint32_t r = 0; r < N; ++r) rank_to_node_.push_back(nodes_[rank[r]].get());
  sequences_.clear();
  for (uint32_t s = 0; s < S; ++s) sequences_.push_back(nodes_[sb[s]].get());
  consensus_.clear();
  for (uint32_t k = 0; k < Cn; ++k) consensus_.push_back(nodes_[cons[k]].get());
  view_valid_ = true;
}

const std::vector<std::unique_ptr<Graph::Node>>& Graph::nodes() const {
  Refresh();
  return nodes_;
}
const std::vector<std::unique_ptr<Graph::Edge>>& Graph::edges() const {
  Refresh();
  return edges_;
}
const std::vector<Graph::Node*>& Graph::rank_to_node() const {
  Refresh();
  return rank_to_node_;
}
const std::vector<Graph::Node*>& Graph::sequences() const {
  Refresh();
  return sequences_;
}
std::uint32_t Graph::num_codes() const {
  Refresh();
  return num_codes_;
}
std::uint8_t Graph::coder(std::uint8_t c) const {
  Refresh();
  return static_cast<std::uint8_t>(coder_[c]);
}
std::uint8_t Graph::decoder(std::uint8_t code) const {
  Refresh();
  return static_cast<std::uint8_t>(decoder_[code]);
}
const std::vector<Graph::Node*>& Graph::consensus() const {
  Refresh();
  return consensus_;
}

void Graph::AddAlignment(const Alignment& alignment, const std::string& sequence,
                         std::uint32_t weight) {
  AddAlignment(alignment, sequence.c_str(), static_cast<std::uint32_t>(sequence.size()), weight);
}

void Graph::AddAlignment(const Alignment& alignment, const std::string& sequence,
                         const std::vector<std::uint32_t>& weights) {
  AddAlignment(alignment, sequence.c_str(), static_cast<std::uint32_t>(sequence.size()), weights);
}

void Graph::AddAlignment(const Alignment& alignment, const std::string& sequence,
                         const std::string& quality) {
  AddAlignment(alignment, sequence.c_str(), static_cast<std::uint32_t>(sequence.size()),
               quality.c_str(), static_cast<std::uint32_t>(quality.size()));
}

void Graph::AddAlignment(const Alignment& alignment, const char* sequence,
                         std::uint32_t sequence_len, std::uint32_t weight) {
  AddAlignment(alignment, sequence, sequence_len,
               std::vector<std::uint32_t>(sequence_len, weight));
}

void Graph::AddAlignment(const Alignment& alignment, const char* sequence,
                         std::uint32_t sequence_len, const std::vector<std::uint32_t>& weights) {
  const std::vector<int32_t> pairs = FlattenAlignment(alignment);
  Invalidate();
  Check("Graph::AddAlignment",
        spoa_gb300_graph_add_alignment(handle_, pairs.data(),
                                       static_cast<uint32_t>(alignment.size()), sequence,
                                       sequence_len, weights.data(),
                                       static_cast<uint32_t>(weights.size())));
}

void Graph::AddAlignment(const Alignment& alignment, const char* sequence,
                         std::uint32_t sequence_len, const char* quality,
                         std::uint32_t quality_len) {
  const std::vector<int32_t> pairs = FlattenAlignment(alignment);
  Invalidate();
  Check("Graph::AddAlignment",
        spoa_gb300_graph_add_alignment_quality(handle_, pairs.data(),
                                               static_cast<uint32_t>(alignment.size()), sequence,
                                               sequence_len, quality, quality_len));
}

std::string Graph::GenerateConsensus() {
  uint32_t N = 0, E = 0, S = 0, Cn = 0, Lb = 0, codes = 0;
  Check("Graph::GenerateConsensus",
        spoa_gb300_graph_counts(handle_, &N, &E, &S, &Cn, &Lb, &codes));
  std::string out(std::max<uint32_t>(N, 1), '\0');
  uint32_t len = 0;
  Invalidate();
  Check("Graph::GenerateConsensus",
        spoa_gb300_graph_consensus(handle_, &out[0], static_cast<uint32_t>(out.size()), &len));
  out.resize(len);
  return out;
}

std::vector<std::string> Graph::GenerateMultipleSequenceAlignment(bool include_consensus) {
  uint32_t N = 0, E = 0, S = 0, Cn = 0, Lb = 0, codes = 0;
  Check("Graph::GenerateMultipleSequenceAlignment",
        spoa_gb300_graph_counts(handle_, &N, &E, &S, &Cn, &Lb, &codes));
  const uint64_t cap = static_cast<uint64_t>(S + 1) * std::max<uint32_t>(N, 1);
  std::vector<char> buf(cap);
  uint32_t rows = 0, cols = 0;
  if (include_consensus) Invalidate();  // the consensus path is regenerated
  Check("Graph::GenerateMultipleSequenceAlignment",
        spoa_gb300_graph_msa(handle_, include_consensus ? 1 : 0, buf.data(), cap, &rows, &cols));
  std::vector<std::string> out;
  out.reserve(rows);
  for (uint32_t r = 0; r < rows; ++r)
    out.emplace_back(buf.data() + static_cast<uint64_t>(r) * cols, cols);
  return out;
}

// Column of every node in the MSA: rank order, aligned groups share one
// column (graph.cpp:321-337).
std::vector<std::uint32_t> Graph::NodeColumns(std::uint32_t* row_size) const {
  Refresh();
  std::vector<std::uint32_t> col(nodes_.size());
  std::uint32_t j = 0;
  for (std::uint32_t i = 0; i < rank_to_node_.size(); ++i, ++j) {
    const Node* it = rank_to_node_[i];
    col[it->id] = j;
    for (const Node* a : it->aligned_nodes) {
      col[a->id] = j;
      ++i;
    }
  }
  if (row_size) *row_size = j;
  return col;
}

std::string Graph::GenerateConsensus(std::vector<std::uint32_t>* summary, bool verbose) {
  if (!summary) Throw("Graph::GenerateConsensus", "invalid ptr to summary");
  std::string dst = GenerateConsensus();
  Refresh();
  summary->clear();
  const std::size_t C = consensus_.size();
  if (!verbose) {
    for (const Node* it : consensus_) {
      std::uint32_t cov = it->Coverage();
      for (const Node* a : it->aligned_nodes) cov += a->Coverage();
      summary->push_back(cov);
    }
    return dst;
  }
  // per consensus column: how many sequences carry each code there, and in
  // the last row how many skip it between two consensus columns they cover
  summary->assign((num_codes_ + 1) * C, 0);
  const std::vector<std::uint32_t> column = NodeColumns(nullptr);
  for (std::uint32_t s = 0; s < sequences_.size(); ++s) {
    const Node* it = sequences_[s];
    std::size_t k = 0, last = 0;
    bool seen = false;
    std::uint32_t col = column[it->id];
    while (true) {
      while (k < C && column[consensus_[k]->id] < col) ++k;
      if (k < C && column[consensus_[k]->id] == col) {
        if (seen)
          for (std::size_t x = last + 1; x < k; ++x) ++(*summary)[num_codes_ * C + x];
        seen = true;
        last = k;
        ++(*summary)[it->code * C + k];
      }
      if (k == C || !(it = it->Successor(s))) break;
      col = column[it->id];
    }
  }
  return dst;
}

Graph Graph::Subgraph(std::uint32_t begin, std::uint32_t end,
                      std::vector<const Node*>* subgraph_to_graph) const {
  if (!subgraph_to_graph) Throw("Graph::Subgraph", "invalid ptr to subgraph_to_graph");
  Refresh();
  const std::size_t n = nodes_.size();
  if (begin >= n || end >= n) Throw("Graph::Subgraph", "invalid node id");
  Graph sub;
  std::vector<uint32_t> map(n);
  Check("Graph::Subgraph", spoa_gb300_graph_subgraph(handle_, begin, end, sub.handle_,
                                                      map.data(), static_cast<uint32_t>(n)));
  subgraph_to_graph->assign(n, nullptr);
  for (std::size_t k = 0; k < n && map[k] != 0xFFFFFFFFu; ++k)
    (*subgraph_to_graph)[k] = nodes_[map[k]].get();
  sub.Invalidate();
  return sub;
}

void Graph::UpdateAlignment(const std::vector<const Node*>& subgraph_to_graph,
                            Alignment* alignment) const {
  for (auto& it : *alignment)
    if (it.first != -1) it.first = static_cast<std::int32_t>(subgraph_to_graph[it.first]->id);
}

void Graph::PrintDot(const std::string& path) const {
  if (path.empty()) return;
  Refresh();
  std::ofstream os(path);
  std::vector<std::int32_t> crank(nodes_.size(), -1);
  std::int32_t r = 0;
  for (const Node* it : consensus_) crank[it->id] = r++;
  os << "digraph " << sequences_.size() << " {\n  graph [rankdir = LR]\n";
  for (const auto& it : nodes_) {
    os << "  " << it->id << "[label = \"" << it->id << " - "
       << static_cast<char>(decoder_[it->code]) << "\"";
    if (crank[it->id] != -1) os << ", style = filled, fillcolor = goldenrod1";
    os << "]\n";
    for (const Edge* e : it->outedges) {
      os << "  " << it->id << " -> " << e->head->id << " [label = \"" << e->weight << "\"";
      if (crank[it->id] + 1 == crank[e->head->id]) os << ", color = goldenrod1";
      os << "]\n";
    }
    for (const Node* a : it->aligned_nodes)
      if (a->id > it->id)
        os << "  " << it->id << " -> " << a->id << " [style = dotted, arrowhead = none]\n";
  }
  os << "}\n";
}

void Graph::Clear() {
  Invalidate();
  Check("Graph::Clear", spoa_gb300_graph_clear(handle_));
}

std::vector<std::uint8_t> Graph::Serialize() const {
  uint64_t n = 0;
  Check("Graph::save", spoa_gb300_graph_save(handle_, nullptr, 0, &n));
  std::vector<std::uint8_t> bytes(n);
  Check("Graph::save", spoa_gb300_graph_save(handle_, bytes.data(), n, &n));
  return bytes;
}

void Graph::Deserialize(const std::vector<std::uint8_t>& bytes) {
  Invalidate();
  // a fresh view: node and edge objects of the old graph are not reused
  nodes_.clear();
  edges_.clear();
  Check("Graph::load", spoa_gb300_graph_load(handle_, bytes.data(), bytes.size()));
}

}  // namespace spoa
