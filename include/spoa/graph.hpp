// spoa/graph.hpp - spoa's partial-order graph, resident on the GPU.
//
// Source-compatible with spoa v4's include/spoa/graph.hpp: the same Node /
// Edge types, accessors, AddAlignment overloads, consensus / MSA calls,
// Subgraph / UpdateAlignment and (under SPOA_USE_CEREAL) cereal save / load
// hooks, whose bytes are this library's own layout.  The graph lives in
// device memory (libspoa_gb300.so); AddAlignment, GenerateConsensus and
// GenerateMultipleSequenceAlignment run there.  The host views returned by
// nodes(), edges(), rank_to_node(), sequences() and consensus() are brought
// up to date from a device export the first time one is read after a
// change.  Nodes and edges are only appended until Clear, and the Node and
// Edge objects of a view are kept and updated by the next one, so pointers
// to them stay valid until Clear, as the reference's do.
#ifndef SPOA_GRAPH_HPP_
#define SPOA_GRAPH_HPP_

#include <cstdint>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#ifdef SPOA_USE_CEREAL
#include "cereal/access.hpp"
#include "cereal/types/vector.hpp"
#endif

struct spoa_gb300_graph;

namespace spoa {

using Alignment = std::vector<std::pair<std::int32_t, std::int32_t>>;

class Graph {
 public:
  Graph();

  Graph(const Graph&) = delete;
  Graph& operator=(const Graph&) = delete;

  Graph(Graph&&) noexcept;
  Graph& operator=(Graph&&) noexcept;

  ~Graph();

  struct Node;
  struct Edge;

  // graph.hpp:40-70 of the reference
  struct Node {
    Node(std::uint32_t id, std::uint32_t code);

    // head of the out-edge carrying sequence `label`, or nullptr
    Node* Successor(std::uint32_t label) const;
    // number of distinct sequence labels on the in- and out-edges
    std::uint32_t Coverage() const;

    std::uint32_t id;
    std::uint32_t code;
    std::vector<Edge*> inedges;
    std::vector<Edge*> outedges;
    std::vector<Node*> aligned_nodes;
  };

  // graph.hpp:72-100 of the reference
  struct Edge {
    Edge(Node* tail, Node* head, std::uint32_t label, std::uint32_t weight);

    void AddSequence(std::uint32_t label, std::uint32_t weight = 1);

    Node* tail;
    Node* head;
    std::vector<std::uint32_t> labels;
    std::int64_t weight;
  };

  const std::vector<std::unique_ptr<Node>>& nodes() const;
  const std::vector<std::unique_ptr<Edge>>& edges() const;
  const std::vector<Node*>& rank_to_node() const;
  const std::vector<Node*>& sequences() const;
  std::uint32_t num_codes() const;
  std::uint8_t coder(std::uint8_t c) const;
  std::uint8_t decoder(std::uint8_t code) const;
  // the last consensus path (empty before GenerateConsensus)
  const std::vector<Node*>& consensus() const;

  // graph.cpp:112-247 of the reference: merge one aligned sequence.  Throws
  // std::invalid_argument with the reference's messages.
  void AddAlignment(const Alignment& alignment, const std::string& sequence,
                    std::uint32_t weight = 1);
  void AddAlignment(const Alignment& alignment, const std::string& sequence,
                    const std::vector<std::uint32_t>& weights);
  void AddAlignment(const Alignment& alignment, const std::string& sequence,
                    const std::string& quality);
  void AddAlignment(const Alignment& alignment, const char* sequence,
                    std::uint32_t sequence_len, std::uint32_t weight = 1);
  void AddAlignment(const Alignment& alignment, const char* sequence,
                    std::uint32_t sequence_len, const std::vector<std::uint32_t>& weights);
  void AddAlignment(const Alignment& alignment, const char* sequence,
                    std::uint32_t sequence_len, const char* quality,
                    std::uint32_t quality_len);

  // graph.cpp:339-366
  std::vector<std::string> GenerateMultipleSequenceAlignment(bool include_consensus = false);

  // graph.cpp:368-375
  std::string GenerateConsensus();

  // graph.cpp:377-431: per consensus base the coverage of its column
  // (verbose: per code and gap row counts)
  std::string GenerateConsensus(std::vector<std::uint32_t>* summary, bool verbose = false);

  // graph.cpp:541-595: the part of the graph that reaches node `end` over
  // in-edges and aligned nodes without going below node id `begin`, as a
  // new graph (sorted, no sequences); subgraph_to_graph gets one entry per
  // node of this graph: this graph's node for each subgraph node, then
  // nullptr.  Throws std::invalid_argument for a null subgraph_to_graph
  // (the reference's message) and for node ids past the graph (which the
  // reference does not check).
  Graph Subgraph(std::uint32_t begin, std::uint32_t end,
                 std::vector<const Node*>* subgraph_to_graph) const;

  // graph.cpp:597-605: maps the node ids of an alignment against a
  // subgraph to this graph's
  void UpdateAlignment(const std::vector<const Node*>& subgraph_to_graph,
                       Alignment* alignment) const;

  // graph.cpp:607-647: Graphviz text of the graph (consensus nodes coloured)
  void PrintDot(const std::string& path) const;

  // graph.cpp:649-658
  void Clear();

  // Persistence.  The reference archives a Graph with cereal
  // (graph.hpp:187-276); here Serialize gives the same fields (coder
  // tables, nodes, edges with labels and weights, sequence starts, aligned
  // pairs, rank order, last consensus) in this library's own byte layout,
  // and Deserialize rebuilds a graph from them the way the reference's load
  // does.  With SPOA_USE_CEREAL, save/load put those bytes into any cereal
  // archive, so archive(graph) works as with the reference.
  std::vector<std::uint8_t> Serialize() const;
  void Deserialize(const std::vector<std::uint8_t>& bytes);
#ifdef SPOA_USE_CEREAL
  template <class Archive>
  void save(Archive& archive) const {  // NOLINT
    archive(Serialize());
  }
  template <class Archive>
  void load(Archive& archive) {  // NOLINT
    std::vector<std::uint8_t> bytes;
    archive(bytes);
    Deserialize(bytes);
  }
#endif

  // The device graph behind this object (for the C ABI and the fused
  // align-and-add call of libspoa_gb300).
  spoa_gb300_graph* device() const { return handle_; }

 private:
  void Invalidate() { view_valid_ = false; }
  void Refresh() const;
  std::vector<std::uint32_t> NodeColumns(std::uint32_t* row_size) const;

  spoa_gb300_graph* handle_;

  // host view, rebuilt on demand
  mutable bool view_valid_;
  mutable std::uint32_t num_codes_;
  mutable std::vector<std::int32_t> coder_;
  mutable std::vector<std::int32_t> decoder_;
  mutable std::vector<std::unique_ptr<Node>> nodes_;
  mutable std::vector<std::unique_ptr<Edge>> edges_;
  mutable std::vector<Node*> rank_to_node_;
  mutable std::vector<Node*> sequences_;
  mutable std::vector<Node*> consensus_;
};

}  // namespace spoa

#endif  // SPOA_GRAPH_HPP_
