// ref_driver.cpp - runs POA windows through the UNMODIFIED reference library.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/Makefile against the reference
// sources (include/ and src/ of the spoa tree) into oracle/_ref/; used to pin
// the C oracle and to generate the golden fixtures under tests/golden/.
//
// It replays the CLI's per-read loop (src/main.cpp:275-314: Align, optional
// strand-ambiguous second strand, AddAlignment with or without qualities)
// and prints, per window, every read's score and alignment, the consensus,
// the MSA rows and the GFA text in the layout of PrintGfa
// (src/main.cpp:119-199).
//
// Input (text, one or more windows):
//   W <type> <m> <n> <g> <e> <q> <c> <strand_ambiguous> <has_quality> <reads>
//   <sequence>            one line per read
//   <quality>             one line per read when has_quality is 1
// Output:
//   W <index>
//   R <read> <score> <reversed> <pairs> <node>,<pos> ...
//   C <consensus>
//   M <msa row>           one per read
//   G <gfa line>          GFA with the consensus path
//   E
// A window that throws prints "X <message>" and continues with the next.
//
// Slice windows (Graph::Subgraph + UpdateAlignment, src/graph.cpp:518-605,
// the way polishers align a read to the part of the graph it spans):
//   S <type> <m> <n> <g> <e> <q> <c> <reads>
//   <sequence>            one line per read; read 0 is added whole
//   <begin> <end>         one line per read after the first: node ids of
//                         the slice (-1 -1: align to the whole graph)
// Output, per read after the first:
//   U <read> <subgraph nodes> <subgraph_to_graph ids ...>
//   K <characters of the subgraph's nodes, in id order>
//   O <subgraph rank_to_node ids>
//   L <tail>,<head>,<weight> ...   subgraph edges in edge order
//   A <node>:<aligned>,... ...     subgraph aligned lists (non-empty ones)
//   Q <subgraph consensus>
//   R <read> <score> 0 <pairs> <node>,<pos> ...   after UpdateAlignment
// then C, M and E as above.
//
// Persisted windows (Graph::save / Graph::load, include/spoa/graph.hpp:
// 187-276, through the archives of ref_shim/cereal):
//   P <type> <m> <n> <g> <e> <q> <c> <has_quality> <reads> <split>
//   <sequence> [<quality>]  per read
// Reads before `split` go into a graph (then GenerateConsensus); it is
// saved and loaded into a second graph, which is printed as loaded
//   K <node characters>   O <rank_to_node ids>   S <sequence start ids>
//   Q <consensus ids>     L <tail>,<head>,<weight>,<label>|<label>... per edge
//   A <node>:<aligned>,... per node with aligned nodes
// and then takes the remaining reads: R lines for them, C, M, G and E.
#include <algorithm>
#include <chrono>
#include <cstdint>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "spoa/spoa.hpp"

namespace {

char Complement(char ch) {
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

void ReverseComplement(std::string* data, std::string* quality) {
  for (auto& ch : *data) ch = Complement(ch);
  std::reverse(data->begin(), data->end());
  std::reverse(quality->begin(), quality->end());
}

void WriteGfa(const spoa::Graph& graph, const std::vector<bool>& is_reversed,
              std::ostream& os) {
  std::vector<bool> is_consensus_node(graph.nodes().size(), false);
  for (const auto& it : graph.consensus()) is_consensus_node[it->id] = true;
  os << "G H\tVN:Z:1.0\n";
  for (const auto& it : graph.nodes()) {
    os << "G S\t" << it->id + 1 << "\t"
       << static_cast<char>(graph.decoder(it->code));
    if (is_consensus_node[it->id]) os << "\tic:Z:true";
    os << "\n";
    for (const auto& jt : it->outedges) {
      os << "G L\t" << it->id + 1 << "\t+\t" << jt->head->id + 1
         << "\t+\tOM\tew:f:" << jt->weight;
      if (is_consensus_node[it->id] && is_consensus_node[jt->head->id]) {
        os << "\tic:Z:true";
      }
      os << "\n";
    }
  }
  for (std::uint32_t i = 0; i < graph.sequences().size(); ++i) {
    os << "G P\tread" << i << "\t";
    std::vector<std::uint32_t> path;
    auto curr = graph.sequences()[i];
    while (curr) {
      path.emplace_back(curr->id + 1);
      curr = curr->Successor(i);
    }
    bool ir = !is_reversed.empty() && is_reversed[i];
    if (ir) std::reverse(path.begin(), path.end());
    for (std::uint32_t j = 0; j < path.size(); ++j) {
      if (j != 0) os << ",";
      os << path[j] << (ir ? "-" : "+");
    }
    os << "\t*\n";
  }
  os << "G P\tConsensus\t";
  for (std::uint32_t i = 0; i < graph.consensus().size(); ++i) {
    if (i != 0) os << ",";
    os << graph.consensus()[i]->id + 1 << "+";
  }
  os << "\t*\n";
}

}  // namespace

int main(int argc, char** argv) {
  bool timing_only = argc > 1 && std::string(argv[1]) == "--time";
  std::string tag;
  std::uint64_t window = 0;
  std::uint64_t cells = 0;
  double seconds = 0;
  while (std::cin >> tag) {
    if (tag == "P") {
      int type, m, n, g, e, q, c, has_quality;
      std::uint32_t reads, split;
      std::cin >> type >> m >> n >> g >> e >> q >> c >> has_quality >> reads >> split;
      std::vector<std::string> data(reads), quality(reads);
      for (std::uint32_t r = 0; r < reads; ++r) {
        std::cin >> data[r];
        if (has_quality) std::cin >> quality[r];
      }
      std::ostringstream os;
      os << "W " << window++ << "\n";
      try {
        auto engine = spoa::AlignmentEngine::Create(
            static_cast<spoa::AlignmentType>(type), m, n, g, e, q, c);
        auto add = [&](spoa::Graph& graph, std::uint32_t r) {
          std::int32_t score = 0;
          auto alignment = engine->Align(data[r], graph, &score);
          if (quality[r].empty()) {
            graph.AddAlignment(alignment, data[r]);
          } else {
            graph.AddAlignment(alignment, data[r], quality[r]);
          }
          return std::make_pair(score, alignment);
        };
        spoa::Graph first{};
        for (std::uint32_t r = 0; r < split; ++r) add(first, r);
        if (split > 0) first.GenerateConsensus();
        std::string bytes;
        cereal::BinaryOutputArchive out(&bytes);
        out(first);
        spoa::Graph graph{};
        cereal::BinaryInputArchive in(bytes);
        in(graph);
        os << "K ";
        for (const auto& it : graph.nodes()) os << static_cast<char>(graph.decoder(it->code));
        os << "\nO";
        for (const auto& it : graph.rank_to_node()) os << " " << it->id;
        os << "\nS";
        for (const auto& it : graph.sequences()) os << " " << it->id;
        os << "\nQ";
        for (const auto& it : graph.consensus()) os << " " << it->id;
        os << "\nL";
        for (const auto& it : graph.edges()) {
          os << " " << it->tail->id << "," << it->head->id << "," << it->weight << ",";
          for (std::size_t k = 0; k < it->labels.size(); ++k) os << (k ? "|" : "") << it->labels[k];
        }
        os << "\nA";
        for (const auto& it : graph.nodes()) {
          if (it->aligned_nodes.empty()) continue;
          os << " " << it->id << ":";
          for (std::size_t k = 0; k < it->aligned_nodes.size(); ++k)
            os << (k ? "," : "") << it->aligned_nodes[k]->id;
        }
        os << "\n";
        for (std::uint32_t r = split; r < reads; ++r) {
          auto res = add(graph, r);
          os << "R " << r << " " << res.first << " 0 " << res.second.size();
          for (const auto& it : res.second) os << " " << it.first << "," << it.second;
          os << "\n";
        }
        os << "C " << graph.GenerateConsensus() << "\n";
        for (const auto& row : graph.GenerateMultipleSequenceAlignment()) os << "M " << row << "\n";
        WriteGfa(graph, std::vector<bool>(), os);
      } catch (std::exception& ex) {
        os << "X " << ex.what() << "\n";
      }
      os << "E\n";
      std::cout << os.str();
      continue;
    }
    if (tag == "S") {
      int type, m, n, g, e, q, c;
      std::uint32_t reads;
      std::cin >> type >> m >> n >> g >> e >> q >> c >> reads;
      std::vector<std::string> data(reads);
      for (std::uint32_t r = 0; r < reads; ++r) std::cin >> data[r];
      std::vector<std::int64_t> lo(reads, -1), hi(reads, -1);
      for (std::uint32_t r = 1; r < reads; ++r) std::cin >> lo[r] >> hi[r];
      std::ostringstream os;
      os << "W " << window++ << "\n";
      try {
        auto engine = spoa::AlignmentEngine::Create(
            static_cast<spoa::AlignmentType>(type), m, n, g, e, q, c);
        spoa::Graph graph{};
        for (std::uint32_t r = 0; r < reads; ++r) {
          std::int32_t score = 0;
          spoa::Alignment alignment;
          if (r > 0 && lo[r] >= 0) {
            std::vector<const spoa::Graph::Node*> map;
            auto sub = graph.Subgraph(static_cast<std::uint32_t>(lo[r]),
                                      static_cast<std::uint32_t>(hi[r]), &map);
            os << "U " << r << " " << sub.nodes().size();
            for (std::size_t k = 0; k < sub.nodes().size(); ++k) os << " " << map[k]->id;
            os << "\nK ";
            for (const auto& it : sub.nodes()) os << static_cast<char>(sub.decoder(it->code));
            os << "\nO";
            for (const auto& it : sub.rank_to_node()) os << " " << it->id;
            os << "\nL";
            for (const auto& it : sub.edges())
              os << " " << it->tail->id << "," << it->head->id << "," << it->weight;
            os << "\nA";
            for (const auto& it : sub.nodes()) {
              if (it->aligned_nodes.empty()) continue;
              os << " " << it->id << ":";
              for (std::size_t k = 0; k < it->aligned_nodes.size(); ++k)
                os << (k ? "," : "") << it->aligned_nodes[k]->id;
            }
            alignment = engine->Align(data[r], sub, &score);
            os << "\nQ " << sub.GenerateConsensus() << "\n";
            graph.UpdateAlignment(map, &alignment);
          } else if (r > 0) {
            alignment = engine->Align(data[r], graph, &score);
          }
          graph.AddAlignment(alignment, data[r]);
          if (r > 0) {
            os << "R " << r << " " << score << " 0 " << alignment.size();
            for (const auto& it : alignment) os << " " << it.first << "," << it.second;
            os << "\n";
          }
        }
        os << "C " << graph.GenerateConsensus() << "\n";
        for (const auto& row : graph.GenerateMultipleSequenceAlignment()) os << "M " << row << "\n";
      } catch (std::exception& ex) {
        os << "X " << ex.what() << "\n";
      }
      os << "E\n";
      std::cout << os.str();
      continue;
    }
    if (tag != "W") return 2;
    int type, m, n, g, e, q, c, strand, has_quality;
    std::uint32_t reads;
    std::cin >> type >> m >> n >> g >> e >> q >> c >> strand >> has_quality >>
        reads;
    std::vector<std::string> data(reads), quality(reads);
    for (std::uint32_t r = 0; r < reads; ++r) {
      std::cin >> data[r];
      if (has_quality) std::cin >> quality[r];
    }
    std::ostringstream os;
    os << "W " << window++ << "\n";
    auto t0 = std::chrono::steady_clock::now();
    try {
      auto engine = spoa::AlignmentEngine::Create(
          static_cast<spoa::AlignmentType>(type), m, n, g, e, q, c);
      spoa::Graph graph{};
      std::vector<bool> is_reversed;
      for (std::uint32_t r = 0; r < reads; ++r) {
        cells += static_cast<std::uint64_t>(graph.nodes().size()) *
                 data[r].size() * (strand ? 2 : 1);
        std::int32_t score = 0;
        auto alignment = engine->Align(data[r], graph, &score);
        bool rev = false;
        if (strand) {
          ReverseComplement(&data[r], &quality[r]);
          std::int32_t score_rev = 0;
          auto alignment_rev = engine->Align(data[r], graph, &score_rev);
          if (score >= score_rev) {
            ReverseComplement(&data[r], &quality[r]);
          } else {
            alignment = alignment_rev;
            score = score_rev;
            rev = true;
          }
          is_reversed.push_back(rev);
        }
        if (quality[r].empty()) {
          graph.AddAlignment(alignment, data[r]);
        } else {
          graph.AddAlignment(alignment, data[r], quality[r]);
        }
        if (!timing_only) {
          os << "R " << r << " " << score << " " << (rev ? 1 : 0) << " "
             << alignment.size();
          for (const auto& it : alignment) {
            os << " " << it.first << "," << it.second;
          }
          os << "\n";
        }
      }
      auto consensus = graph.GenerateConsensus();
      if (!timing_only) {
        os << "C " << consensus << "\n";
        // per-base support (graph.cpp:377-431), both forms
        for (int verbose = 0; verbose < 2; ++verbose) {
          std::vector<std::uint32_t> summary;
          graph.GenerateConsensus(&summary, verbose != 0);
          os << (verbose ? "V" : "Y");
          for (std::size_t k = 0; k < summary.size(); ++k) os << (k ? "," : " ") << summary[k];
          os << "\n";
        }
        auto msa = graph.GenerateMultipleSequenceAlignment();
        for (const auto& row : msa) os << "M " << row << "\n";
        WriteGfa(graph, is_reversed, os);
      }
    } catch (std::exception& ex) {
      os << "X " << ex.what() << "\n";
    }
    seconds += std::chrono::duration<double>(
        std::chrono::steady_clock::now() - t0).count();
    os << "E\n";
    if (!timing_only) std::cout << os.str();
  }
  if (timing_only) {
    std::cout << "T " << window << " " << cells << " " << seconds << "\n";
  }
  return 0;
}
