// spoa_cli.cpp - the `spoa` command-line program over the GPU library.
//
// A drop-in for the reference CLI (src/main.cpp): the same options (-m -n
// -g -e -q -c, -l/--algorithm, -r/--result repeated, -d/--dot,
// -s/--strand-ambiguous, --version, -h/--help), the same input formats
// (FASTA/FASTQ by file extension, optionally gzip-compressed, names cut at
// the first whitespace as bioparser 3.0.13 cuts them) and the same output
// bytes: consensus and MSA as FASTA, the graph as GFA 1.0 (main.cpp:119-199)
// and as DOT (Graph::PrintDot).  Each read of the loop (main.cpp:275-314,
// strand choice of main.cpp:285-302 included) is one spoa_gb300_align_add
// call: align and add fused on the device, the alignment never leaves it,
// and the DP arena grows with the graph as the reference's does.
#include <getopt.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#if __has_include(<zlib.h>)
#include <zlib.h>
#define SPOA_CLI_HAS_ZLIB 1
#else
#define SPOA_CLI_HAS_ZLIB 0
#endif

#include "spoa/spoa.hpp"
#include "spoa_gb300.h"

namespace {

const char* kVersion = "4.0.8";  // the spoa release whose interface this mirrors

struct Record {
  std::string name, data, quality;
};

// Line reader over a plain or gzip file (zlib reads both).
class LineFile {
 public:
  explicit LineFile(const std::string& path) {
#if SPOA_CLI_HAS_ZLIB
    gz_ = gzopen(path.c_str(), "r");
#else
    const bool gz = path.size() > 3 && path.compare(path.size() - 3, 3, ".gz") == 0;
    f_ = gz ? nullptr : std::fopen(path.c_str(), "r");
#endif
  }
  ~LineFile() {
#if SPOA_CLI_HAS_ZLIB
    if (gz_) gzclose(gz_);
#else
    if (f_) std::fclose(f_);
#endif
  }
  bool ok() const {
#if SPOA_CLI_HAS_ZLIB
    return gz_ != nullptr;
#else
    return f_ != nullptr;
#endif
  }
  // next line without its end and trailing blanks; false at end of file
  bool Next(std::string* line) {
    line->clear();
    bool any = false;
    for (;;) {
#if SPOA_CLI_HAS_ZLIB
      const int ch = gzgetc(gz_);
#else
      const int ch = std::fgetc(f_);
#endif
      if (ch < 0) break;
      any = true;
      if (ch == '\n') break;
      line->push_back(static_cast<char>(ch));
    }
    const auto keep = line->find_last_not_of(" \t\r");
    line->resize(keep == std::string::npos ? 0 : keep + 1);
    return any;
  }

 private:
#if SPOA_CLI_HAS_ZLIB
  gzFile gz_ = nullptr;
#else
  FILE* f_ = nullptr;
#endif
};

std::string ShortName(const std::string& header) {
  std::string n = header.substr(1);
  const auto k = n.find_first_of(" \t");
  if (k != std::string::npos) n.resize(k);
  return n;
}

// FASTA: '>' header, data lines up to the next header, concatenated.
void ReadFasta(LineFile* in, std::vector<Record>* out) {
  std::string line;
  bool open = false;
  auto close = [&]() {
    if (open && (out->back().name.empty() || out->back().data.empty()))
      throw std::invalid_argument("[bioparser::FastaParser] error: invalid file format");
  };
  while (in->Next(&line)) {
    if (line.empty()) continue;
    if (line[0] == '>') {
      close();
      out->push_back({ShortName(line), "", ""});
      open = true;
    } else if (open) {
      out->back().data += line;
    } else {
      throw std::invalid_argument("[bioparser::FastaParser] error: invalid file format");
    }
  }
  close();
}

// FASTQ: '@' header, sequence lines up to a '+' line, quality lines until
// the quality is as long as the sequence.
void ReadFastq(LineFile* in, std::vector<Record>* out) {
  const std::invalid_argument bad("[bioparser::FastqParser] error: invalid file format");
  std::string line;
  while (in->Next(&line)) {
    if (line.empty()) continue;
    if (line[0] != '@') throw bad;
    Record r{ShortName(line), "", ""};
    bool plus = false;
    while (in->Next(&line)) {
      if (!line.empty() && line[0] == '+') {
        plus = true;
        break;
      }
      r.data += line;
    }
    if (!plus) throw bad;
    while (r.quality.size() < r.data.size() && in->Next(&line)) r.quality += line;
    if (r.name.empty() || r.data.empty() || r.quality.size() != r.data.size()) throw bad;
    out->push_back(std::move(r));
  }
}

bool EndsWith(const std::string& s, const char* suffix) {
  const std::string t(suffix);
  return s.size() >= t.size() && s.compare(s.size() - t.size(), t.size(), t) == 0;
}

// 0: FASTA, 1: FASTQ, -1: unsupported extension (main.cpp:25-59)
int FormatOf(const std::string& path) {
  for (const char* x : {".fasta", ".fna", ".faa", ".fa"})
    if (EndsWith(path, x) || EndsWith(path, (std::string(x) + ".gz").c_str())) return 0;
  for (const char* x : {".fastq", ".fq"})
    if (EndsWith(path, x) || EndsWith(path, (std::string(x) + ".gz").c_str())) return 1;
  return -1;
}

void Usage() {
  std::cout <<
      "usage: spoa [options ...] <sequences>\n"
      "\n"
      "  partial order alignment of the sequences on the GPU; the result goes\n"
      "  to stdout\n"
      "  <sequences>\n"
      "    FASTA or FASTQ file, plain or gzip-compressed\n"
      "\n"
      "  options:\n"
      "    -m <int>                 match score (default 5)\n"
      "    -n <int>                 mismatch score (default -4)\n"
      "    -g <int>                 gap open, <= 0 (default -8)\n"
      "    -e <int>                 gap extend, <= 0 (default -6)\n"
      "    -q <int>                 second gap open, <= 0 (default -10)\n"
      "    -c <int>                 second gap extend, <= 0 (default -4)\n"
      "    -l, --algorithm <int>    0 local (Smith-Waterman, default),\n"
      "                             1 global (Needleman-Wunsch), 2 semi-global\n"
      "    -r, --result <int>       repeatable; 0 consensus (FASTA, default),\n"
      "                             1 MSA (FASTA), 2 MSA with consensus (FASTA),\n"
      "                             3 graph (GFA), 4 graph with consensus (GFA)\n"
      "    -d, --dot <file>         also write the graph in DOT format\n"
      "    -s, --strand-ambiguous   align both strands, keep the better\n"
      "    --version                print the version\n"
      "    -h, --help               print this text\n"
      "\n"
      "  gaps: linear if g >= e, affine if g <= q or e >= c, convex otherwise\n";
}

// GFA 1.0 in the layout of main.cpp:119-199: S and L lines per node in id
// order (consensus nodes and edges between them tagged ic:Z:true), a P line
// per sequence (reversed paths walked backwards with '-'), and the
// consensus path when asked.
void WriteGfa(const spoa::Graph& graph, const std::vector<std::string>& names,
              const std::vector<bool>& reversed, bool with_consensus) {
  const auto& nodes = graph.nodes();
  std::vector<bool> in_cons(nodes.size(), false);
  for (const auto* n : graph.consensus()) in_cons[n->id] = true;
  std::cout << "H\tVN:Z:1.0\n";
  for (const auto& n : nodes) {
    std::cout << "S\t" << n->id + 1 << "\t" << static_cast<char>(graph.decoder(n->code))
              << (in_cons[n->id] ? "\tic:Z:true" : "") << "\n";
    for (const auto* e : n->outedges) {
      std::cout << "L\t" << n->id + 1 << "\t+\t" << e->head->id + 1 << "\t+\tOM\tew:f:"
                << e->weight << (in_cons[n->id] && in_cons[e->head->id] ? "\tic:Z:true" : "")
                << "\n";
    }
  }
  const auto& seqs = graph.sequences();
  for (std::uint32_t s = 0; s < seqs.size(); ++s) {
    std::vector<std::uint32_t> path;
    for (const spoa::Graph::Node* it = seqs[s]; it; it = it->Successor(s))
      path.push_back(it->id + 1);
    const bool rev = !reversed.empty() && reversed[s];
    if (rev) std::reverse(path.begin(), path.end());
    std::cout << "P\t" << names[s] << "\t";
    for (std::size_t k = 0; k < path.size(); ++k)
      std::cout << (k ? "," : "") << path[k] << (rev ? "-" : "+");
    std::cout << "\t*\n";
  }
  if (with_consensus) {
    std::cout << "P\tConsensus\t";
    const auto& cons = graph.consensus();
    for (std::size_t k = 0; k < cons.size(); ++k) std::cout << (k ? "," : "") << cons[k]->id + 1 << "+";
    std::cout << "\t*\n";
  }
}

// Where spoa would have thrown for a status of the per-read loop.
std::string LoopError(int32_t st) {
  const bool graph_side = st == SPOA_GB300_ERR_INVALID_ALIGNMENT ||
                          st == SPOA_GB300_ERR_MISSING_SEQUENCE ||
                          st == SPOA_GB300_ERR_UNEQUAL_WEIGHTS;
  return std::string(graph_side ? "[spoa::Graph::AddAlignment]"
                                : "[spoa::CudaAlignmentEngine::Align]") +
         " error: " + spoa_gb300_status_string(st);
}

int Run(int argc, char** argv) {
  int m = 5, n = -4, g = -8, e = -6, q = -10, c = -4, algorithm = 0;
  std::vector<int> results;  // values pass through uint8, as the reference's do
  std::string dot;
  bool strand = false;
  const option longs[] = {{"algorithm", required_argument, nullptr, 'l'},
                          {"result", required_argument, nullptr, 'r'},
                          {"dot", required_argument, nullptr, 'd'},
                          {"strand-ambiguous", no_argument, nullptr, 's'},
                          {"version", no_argument, nullptr, 'v'},
                          {"help", no_argument, nullptr, 'h'},
                          {nullptr, 0, nullptr, 0}};
  int opt;
  while ((opt = getopt_long(argc, argv, "m:n:g:e:q:c:l:r:d:sh", longs, nullptr)) != -1) {
    switch (opt) {
      case 'm': m = std::atoi(optarg); break;
      case 'n': n = std::atoi(optarg); break;
      case 'g': g = std::atoi(optarg); break;
      case 'e': e = std::atoi(optarg); break;
      case 'q': q = std::atoi(optarg); break;
      case 'c': c = std::atoi(optarg); break;
      case 'l': algorithm = std::atoi(optarg); break;
      case 'r': results.push_back(static_cast<std::uint8_t>(std::atoi(optarg))); break;
      case 'd': dot = optarg; break;
      case 's': strand = true; break;
      case 'v': std::cout << kVersion << std::endl; return 0;
      case 'h': Usage(); return 0;
      default: return 1;
    }
  }
  if (results.empty()) results.push_back(0);
  if (optind >= argc) {
    std::cerr << "[spoa::] error: missing input file!" << std::endl;
    Usage();
    return 1;
  }
  const std::string path = argv[optind];
  const int format = FormatOf(path);
  if (format < 0) {
    std::cerr << "[spoa::CreateParser] error: file " << path
              << " has unsupported format extension (valid extensions: .fasta, .fasta.gz, "
                 ".fna, .fna.gz, .faa, .faa.gz, .fa, .fa.gz, .fastq, .fastq.gz, .fq, .fq.gz)"
              << std::endl;
    return 1;
  }
  LineFile in(path);
  if (!in.ok()) {
    std::cerr << "[bioparser::Parser::Create] error: unable to open file " << path << std::endl;
    return 1;
  }
  // the penalties pass through int8, as the reference's options do
  const auto i8 = [](int v) { return static_cast<std::int8_t>(v); };
  std::uint32_t max_len = 0;
  std::vector<Record> reads;
  try {
    // checks and messages of AlignmentEngine::Create (alignment_engine.cpp:32-73)
    spoa::AlignmentEngine::Create(static_cast<spoa::AlignmentType>(static_cast<std::uint8_t>(algorithm)),
                                  i8(m), i8(n), i8(g), i8(e), i8(q), i8(c));
    if (format == 0)
      ReadFasta(&in, &reads);
    else
      ReadFastq(&in, &reads);
    for (const auto& r : reads) max_len = std::max<std::uint32_t>(max_len, r.data.size());
  } catch (std::invalid_argument& ex) {
    std::cerr << ex.what() << std::endl;
    return 1;
  }

  spoa_gb300_engine* engine = nullptr;
  int32_t st = spoa_gb300_engine_create(static_cast<std::uint8_t>(algorithm), i8(m), i8(n), i8(g),
                                        i8(e), i8(q), i8(c), &engine);
  if (st == SPOA_GB300_OK) st = spoa_gb300_engine_prealloc(engine, max_len, 4);
  if (st != SPOA_GB300_OK) {
    std::cerr << "[spoa::CudaAlignmentEngine::Prealloc] error: " << spoa_gb300_status_string(st)
              << std::endl;
    spoa_gb300_engine_destroy(engine);
    return 1;
  }
  std::unique_ptr<spoa_gb300_engine, void (*)(spoa_gb300_engine*)> owner(
      engine, spoa_gb300_engine_destroy);

  spoa::Graph graph{};
  const std::size_t nr = reads.size();
  std::vector<bool> is_reversed;
  for (const auto& rd : reads) {
    int32_t score = 0, rev = 0;
    st = spoa_gb300_align_add(engine, graph.device(), rd.data.data(),
                              static_cast<uint32_t>(rd.data.size()),
                              format == 1 ? rd.quality.data() : nullptr, strand ? 1 : 0, &score,
                              &rev);
    if (st != SPOA_GB300_OK) {
      std::cerr << LoopError(st) << std::endl;
      return 1;
    }
    if (strand) is_reversed.push_back(rev != 0);
  }

  for (int r : results) {
    if (r == 0) {
      const std::string cons = graph.GenerateConsensus();
      std::cout << ">Consensus LN:i:" << cons.size() << "\n" << cons << "\n";
    } else if (r == 1 || r == 2) {
      const auto msa = graph.GenerateMultipleSequenceAlignment(r == 2);
      for (std::size_t k = 0; k < msa.size(); ++k)
        std::cout << ">" << (k < nr ? reads[k].name : std::string("Consensus")) << "\n"
                  << msa[k] << "\n";
    } else if (r == 3 || r == 4) {
      std::vector<std::string> names;
      for (const auto& rd : reads) names.push_back(rd.name);
      graph.GenerateConsensus();
      WriteGfa(graph, names, is_reversed, r == 4);
    }
  }
  std::cout.flush();
  graph.PrintDot(dot);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  try {
    return Run(argc, argv);
  } catch (std::exception& ex) {
    std::cerr << ex.what() << std::endl;
    return 1;
  }
}
