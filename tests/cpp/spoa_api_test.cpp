// spoa_api_test.cpp - drives the C++ API (include/spoa/*.hpp) the way spoa's
// own tests do (test/spoa_test.cpp): Prealloc, Align + AddAlignment of every
// read, GenerateConsensus, GenerateMultipleSequenceAlignment with its
// invariants, Clear and re-run, and the error messages.  Built by
// spoa_gb300.build next to libspoa.so; run by tests/test_cpp_api.py, which
// compares the printed consensus, MSA and summaries with the fixtures.
//
// usage: spoa_api_test <reads.tsv> <cases.txt> [slices.txt]
//   reads.tsv: one read per line, "sequence<TAB>quality"
//   cases.txt: one case per line, "name type m n g e q c quality(0|1)"
//   slices.txt: backbone windows for Graph::Subgraph / UpdateAlignment,
//     "S type m n g e q c reads", the reads, then "begin end" per read after
//     the first (-1 -1: the whole graph); printed as "SLICE <window> R
//     <read> <score> <node,pos ...>" per read and "SLICE <window> C
//     <consensus>"
// Output lines: "CONS <name> <consensus>", "MSA <name> <row>" per row,
// "SUMMARY <name> <v0,v1,...>" and "VSUMMARY" (verbose), "CLEAR <name>
// <ok|mismatch>", "FAIL <what>",
// "ERR <check> <message>", and "DONE <failures>" last.
#include <algorithm>
#include <cstdint>
#include <fstream>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "spoa/spoa.hpp"

namespace {

struct Read {
  std::string data, quality;
};

int failures = 0;

void Fail(const std::string& what) {
  ++failures;
  std::cout << "FAIL " << what << "\n";
}

void AlignAll(spoa::AlignmentEngine& ae, spoa::Graph& gr, const std::vector<Read>& reads,
              bool with_quality) {
  std::size_t longest = 0;
  for (const auto& r : reads) longest = std::max(longest, r.data.size());
  ae.Prealloc(static_cast<std::uint32_t>(longest), 4);
  for (const auto& r : reads) {
    auto a = ae.Align(r.data, gr);
    if (with_quality)
      gr.AddAlignment(a, r.data, r.quality);
    else
      gr.AddAlignment(a, r.data);
  }
}

// The MSA invariants of spoa_test.cpp:56-78: one row per read, equal row
// lengths, no all-gap column, each row without gaps is the read.
void CheckMsa(const std::string& name, const std::vector<std::string>& msa,
              const std::vector<Read>& reads) {
  if (msa.size() != reads.size()) return Fail(name + " msa rows");
  const std::size_t rs = msa.front().size();
  std::vector<std::size_t> gaps(rs, 0);
  for (const auto& row : msa) {
    if (row.size() != rs) return Fail(name + " msa row length");
    for (std::size_t i = 0; i < rs; ++i) gaps[i] += row[i] == '-';
  }
  for (std::size_t g : gaps)
    if (g >= msa.size()) return Fail(name + " all-gap column");
  for (std::size_t i = 0; i < msa.size(); ++i) {
    std::string s = msa[i];
    s.erase(std::remove(s.begin(), s.end(), '-'), s.end());
    if (s != reads[i].data) return Fail(name + " msa row is not the read");
  }
}

// Read 0 added whole; each later read aligned to Subgraph(begin, end) (or
// the whole graph), its alignment mapped back with UpdateAlignment, added.
void RunSlices(const char* path) {
  std::ifstream in(path);
  std::string tag;
  int window = 0;
  while (in >> tag && tag == "S") {
    int type, m, n, g, e, q, c;
    std::uint32_t nr;
    in >> type >> m >> n >> g >> e >> q >> c >> nr;
    std::vector<std::string> reads(nr);
    for (auto& r : reads) in >> r;
    auto ae = spoa::AlignmentEngine::Create(static_cast<spoa::AlignmentType>(type), m, n, g, e,
                                            q, c);
    spoa::Graph gr{};
    gr.AddAlignment(spoa::Alignment(), reads[0]);
    for (std::uint32_t r = 1; r < nr; ++r) {
      long long b, en;
      in >> b >> en;
      std::int32_t score = 0;
      spoa::Alignment a;
      if (b >= 0) {
        std::vector<const spoa::Graph::Node*> map;
        spoa::Graph sub = gr.Subgraph(static_cast<std::uint32_t>(b),
                                      static_cast<std::uint32_t>(en), &map);
        if (map.size() != gr.nodes().size()) Fail("subgraph_to_graph size");
        for (std::size_t k = 0; k < map.size(); ++k)
          if ((k < sub.nodes().size()) != (map[k] != nullptr)) Fail("subgraph_to_graph entry");
        a = ae->Align(reads[r], sub, &score);
        gr.UpdateAlignment(map, &a);
      } else {
        a = ae->Align(reads[r], gr, &score);
      }
      gr.AddAlignment(a, reads[r]);
      std::cout << "SLICE " << window << " R " << r << " " << score;
      for (const auto& it : a) std::cout << " " << it.first << "," << it.second;
      std::cout << "\n";
    }
    std::cout << "SLICE " << window++ << " C " << gr.GenerateConsensus() << "\n";
  }
  // graph.cpp:544-548
  spoa::Graph gr{};
  gr.AddAlignment(spoa::Alignment(), "ACGT");
  try {
    gr.Subgraph(0, 3, nullptr);
    Fail("Subgraph without a map did not throw");
  } catch (std::invalid_argument& ex) {
    std::cout << "ERR SubgraphNullMap " << ex.what() << "\n";
  }
  // node objects outlive later changes of the graph (graph.hpp:40-70)
  const spoa::Graph::Node* first = gr.nodes()[0].get();
  gr.AddAlignment(spoa::Alignment(), "TTTT");
  if (gr.nodes()[0].get() != first || first->id != 0) Fail("node pointer after AddAlignment");
  // persistence: Serialize / Deserialize round trip (graph.hpp:187-276)
  const std::string cons = gr.GenerateConsensus();
  const auto bytes = gr.Serialize();
  spoa::Graph back{};
  back.Deserialize(bytes);
  if (back.nodes().size() != gr.nodes().size() || back.edges().size() != gr.edges().size() ||
      back.sequences().size() != 2 || back.consensus().size() != cons.size() ||
      back.Serialize() != bytes || back.GenerateConsensus() != cons)
    Fail("Serialize / Deserialize round trip");
  std::cout << "ERR Persist ok\n";
}

std::string Join(const std::vector<std::uint32_t>& v) {
  std::ostringstream os;
  for (std::size_t i = 0; i < v.size(); ++i) os << (i ? "," : "") << v[i];
  return os.str();
}

void ErrorChecks() {
  // spoa_test.cpp:86-94
  try {
    auto ae = spoa::AlignmentEngine::Create(static_cast<spoa::AlignmentType>(4), 1, -1, -1);
    Fail("TypeError did not throw");
  } catch (std::invalid_argument& ex) {
    std::cout << "ERR TypeError " << ex.what() << "\n";
  }
  // spoa_test.cpp:96-101
  {
    auto ae = spoa::AlignmentEngine::Create(spoa::AlignmentType::kSW, 1, -1, -1);
    spoa::Graph g{};
    auto a = ae->Align("", g);
    std::cout << "ERR EmptyInput " << (a.empty() ? "empty" : "not-empty") << "\n";
  }
  // spoa_test.cpp:103-118: the text after "[spoa::" and the 4-letter engine
  // prefix
  {
    auto ae = spoa::AlignmentEngine::Create(spoa::AlignmentType::kSW, 1, -1, -1);
    try {
      ae->Prealloc(static_cast<std::uint32_t>(-1), 1);
      Fail("LargeInput too large did not throw");
    } catch (std::invalid_argument& ex) {
      std::cout << "ERR LargeInput1 " << std::string(ex.what()).substr(11) << "\n";
    }
    // with these penalties the worst case overflows even int32, so the
    // reference returns before sizing anything (implementation.hpp:392-397)
    try {
      ae->Prealloc((1ULL << 31) - 1, static_cast<std::uint8_t>(-1));
      std::cout << "ERR LargeInput2 no-throw\n";
    } catch (std::invalid_argument& ex) {
      std::cout << "ERR LargeInput2 " << std::string(ex.what()).substr(11) << "\n";
    }
  }
  // graph.cpp:162-194
  {
    spoa::Graph g{};
    try {
      g.AddAlignment(spoa::Alignment(), "ACGT", std::vector<std::uint32_t>{1, 2});
      Fail("unequal weights did not throw");
    } catch (std::invalid_argument& ex) {
      std::cout << "ERR UnequalWeights " << ex.what() << "\n";
    }
  }
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) {
    std::cerr << "usage: spoa_api_test <reads.tsv> <cases.txt>\n";
    return 2;
  }
  std::vector<Read> reads;
  {
    std::ifstream in(argv[1]);
    std::string line;
    while (std::getline(in, line)) {
      if (line.empty()) continue;
      const auto tab = line.find('\t');
      reads.push_back({line.substr(0, tab), tab == std::string::npos ? "" : line.substr(tab + 1)});
    }
  }
  std::ifstream cases(argv[2]);
  std::string name;
  int type, m, n, g, e, q, c, quality;
  try {
    while (cases >> name >> type >> m >> n >> g >> e >> q >> c >> quality) {
      auto ae = spoa::AlignmentEngine::Create(static_cast<spoa::AlignmentType>(type), m, n, g,
                                              e, q, c);
      spoa::Graph gr{};
      AlignAll(*ae, gr, reads, quality != 0);
      const std::string cons = gr.GenerateConsensus();
      std::cout << "CONS " << name << " " << cons << "\n";
      auto msa = gr.GenerateMultipleSequenceAlignment();
      CheckMsa(name, msa, reads);
      for (const auto& row : msa) std::cout << "MSA " << name << " " << row << "\n";
      std::vector<std::uint32_t> summary;
      gr.GenerateConsensus(&summary, false);
      std::cout << "SUMMARY " << name << " " << Join(summary) << "\n";
      gr.GenerateConsensus(&summary, true);
      std::cout << "VSUMMARY " << name << " " << Join(summary) << "\n";
      // host views: one node per consensus base, consistent edges
      if (gr.consensus().size() != cons.size()) Fail(name + " consensus view");
      std::size_t edges = 0;
      for (const auto& node : gr.nodes()) edges += node->outedges.size();
      if (edges != gr.edges().size()) Fail(name + " edge view");
      if (gr.sequences().size() != reads.size()) Fail(name + " sequences view");
      // spoa_test.cpp:125-130: Clear and align again
      gr.Clear();
      AlignAll(*ae, gr, reads, quality != 0);
      std::cout << "CLEAR " << name << " " << (gr.GenerateConsensus() == cons ? "ok" : "mismatch")
                << "\n";
    }
    ErrorChecks();
    if (argc > 3) RunSlices(argv[3]);
  } catch (std::exception& ex) {
    Fail(std::string("exception: ") + ex.what());
  }
  std::cout << "DONE " << failures << "\n";
  return failures ? 1 : 0;
}
