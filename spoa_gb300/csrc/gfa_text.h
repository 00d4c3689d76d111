// gfa_text.h - GFA 1.0 text of a POA graph from its exported arrays, in the
// layout of the reference CLI's PrintGfa (src/main.cpp:119-199): an H line;
// per node in id order an S line (1-based id, character, ic:Z:true on
// consensus nodes) and its L lines in out-edge order (ew:f:<weight>,
// ic:Z:true when both ends are consensus nodes); per sequence a P line along
// its labelled path (Node::Successor, graph.cpp:22-30), reversed with '-'
// for reads kept on the reverse strand; optionally the Consensus P line.
// Host code over plain arrays (the shape spoa_gb300_graph_export fills).
#pragma once

#include <algorithm>
#include <cstdint>
#include <string>
#include <vector>

namespace spoa_gb300 {

struct GfaGraph {
  uint32_t n_nodes, n_seqs, n_consensus;
  const uint8_t* chars;         // decoded character per node
  const uint32_t *out_off, *out_edges;  // out-edge CSR (edge ids, insertion order)
  const uint32_t* e_head;
  const int64_t* e_weight;
  const uint32_t *label_off, *labels;   // labels of edge e (sequence ids, ascending)
  const uint32_t* seq_begin;
  const uint32_t* consensus;
};

inline std::string gfa_text(const GfaGraph& g, const char* const* headers,
                            const uint8_t* is_reversed, bool include_consensus) {
  std::vector<uint8_t> in_cons(g.n_nodes, 0);
  for (uint32_t k = 0; k < g.n_consensus; ++k) in_cons[g.consensus[k]] = 1;
  std::string s = "H\tVN:Z:1.0\n";
  for (uint32_t v = 0; v < g.n_nodes; ++v) {
    s += "S\t" + std::to_string(v + 1) + "\t" + static_cast<char>(g.chars[v]);
    if (in_cons[v]) s += "\tic:Z:true";
    s += "\n";
    for (uint32_t k = g.out_off[v]; k < g.out_off[v + 1]; ++k) {
      const uint32_t e = g.out_edges[k], h = g.e_head[e];
      s += "L\t" + std::to_string(v + 1) + "\t+\t" + std::to_string(h + 1) + "\t+\tOM\tew:f:" +
           std::to_string(g.e_weight[e]);
      if (in_cons[v] && in_cons[h]) s += "\tic:Z:true";
      s += "\n";
    }
  }
  auto successor = [&](uint32_t v, uint32_t label) -> int64_t {
    for (uint32_t k = g.out_off[v]; k < g.out_off[v + 1]; ++k) {
      const uint32_t e = g.out_edges[k];
      for (uint32_t l = g.label_off[e]; l < g.label_off[e + 1]; ++l)
        if (g.labels[l] == label) return g.e_head[e];
    }
    return -1;
  };
  std::vector<uint32_t> path;
  for (uint32_t sq = 0; sq < g.n_seqs; ++sq) {
    path.clear();
    for (int64_t v = g.seq_begin[sq]; v >= 0 && path.size() <= g.n_nodes; v = successor((uint32_t)v, sq))
      path.push_back((uint32_t)v + 1);
    const bool rev = is_reversed && is_reversed[sq];
    if (rev) std::reverse(path.begin(), path.end());
    s += "P\t";
    s += headers ? std::string(headers[sq]) : "read" + std::to_string(sq);
    s += "\t";
    for (size_t k = 0; k < path.size(); ++k) {
      if (k) s += ",";
      s += std::to_string(path[k]) + (rev ? "-" : "+");
    }
    s += "\t*\n";
  }
  if (include_consensus) {
    s += "P\tConsensus\t";
    for (uint32_t k = 0; k < g.n_consensus; ++k) {
      if (k) s += ",";
      s += std::to_string(g.consensus[k] + 1) + "+";
    }
    s += "\t*\n";
  }
  return s;
}

}  // namespace spoa_gb300
