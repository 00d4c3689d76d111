// ref_bench.cpp - times the UNMODIFIED reference library on host threads.
//
// TEST INFRASTRUCTURE ONLY (the CPU baseline of bench.py).  Built by
// oracle/Makefile (target `bench`) against the reference's own library
// sources into oracle/_ref/.  On an x86 host with AVX2 the reference builds
// its SimdAlignmentEngine; on other hosts (the aarch64 GPU machine) its
// AlignmentEngine::Create falls back to the SisdAlignmentEngine
// (src/alignment_engine.cpp:68-72), which is the reference's real CPU path
// there.
//
// The way spoa's callers run many windows: one window per task on a pool of
// threads, each thread with its own AlignmentEngine (one per alignment type,
// Prealloc'd once like src/main.cpp:265-271) and a fresh Graph per window;
// per read Align, for strand-ambiguous windows also the reverse complement
// (keep the forward strand if score >= score_rev, src/main.cpp:285-302),
// AddAlignment; then GenerateConsensus.
//
// Input (binary, little-endian): "SPWB", u32 n_windows, then per window
//   i8 type, i8 strand_ambiguous, u16 0, u32 n_reads, n_reads x u32 length,
//   the reads' bytes back to back.
// Usage: spoa_ref_bench <input> <m> <n> <g> <e> <q> <c> <threads> [<consensus out>]
// Prints one JSON line: windows, seconds (wall, all threads), threads, DP
// cells (read length x graph nodes per Align call), per-window seconds
// p50/p99, engine ("simd" or "sisd" build).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "spoa/spoa.hpp"

namespace {

struct Window {
  int type = 0;
  bool strand = false;
  std::vector<std::string> reads;
};

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

std::string ReverseComplement(const std::string& s) {
  std::string r(s.rbegin(), s.rend());
  for (auto& ch : r) ch = Complement(ch);
  return r;
}

template <typename T>
bool Get(std::ifstream& in, T* v) {
  return static_cast<bool>(in.read(reinterpret_cast<char*>(v), sizeof(T)));
}

bool Load(const char* path, std::vector<Window>* out) {
  std::ifstream in(path, std::ios::binary);
  char magic[4];
  uint32_t n = 0;
  if (!in.read(magic, 4) || std::memcmp(magic, "SPWB", 4) != 0 || !Get(in, &n)) return false;
  out->resize(n);
  for (auto& w : *out) {
    int8_t type = 0, strand = 0;
    uint16_t pad = 0;
    uint32_t nr = 0;
    if (!Get(in, &type) || !Get(in, &strand) || !Get(in, &pad) || !Get(in, &nr)) return false;
    w.type = type;
    w.strand = strand != 0;
    std::vector<uint32_t> lens(nr);
    for (auto& l : lens)
      if (!Get(in, &l)) return false;
    w.reads.resize(nr);
    for (uint32_t r = 0; r < nr; ++r) {
      w.reads[r].resize(lens[r]);
      if (lens[r] && !in.read(&w.reads[r][0], lens[r])) return false;
    }
  }
  return true;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 9) {
    std::cerr << "usage: spoa_ref_bench <input> <m> <n> <g> <e> <q> <c> <threads> [<out>]\n";
    return 1;
  }
  std::vector<Window> wins;
  if (!Load(argv[1], &wins)) {
    std::cerr << "cannot read " << argv[1] << "\n";
    return 1;
  }
  int8_t p[6];
  for (int k = 0; k < 6; ++k) p[k] = static_cast<int8_t>(std::atoi(argv[2 + k]));
  const int threads = std::max(1, std::atoi(argv[8]));
  uint32_t max_len = 1;
  for (const auto& w : wins)
    for (const auto& r : w.reads) max_len = std::max<uint32_t>(max_len, r.size());

  std::vector<std::string> consensus(wins.size());
  std::vector<double> secs(wins.size(), 0.0);
  std::atomic<uint32_t> next{0};
  std::atomic<uint64_t> cells{0};
  std::atomic<int> failed{0};
  auto worker = [&]() {
    std::unique_ptr<spoa::AlignmentEngine> engines[3];
    uint64_t my_cells = 0;
    try {
      while (true) {
        const uint32_t w = next++;
        if (w >= wins.size()) break;
        const Window& win = wins[w];
        auto& engine = engines[win.type];
        if (!engine) {
          engine = spoa::AlignmentEngine::Create(static_cast<spoa::AlignmentType>(win.type),
                                                 p[0], p[1], p[2], p[3], p[4], p[5]);
          engine->Prealloc(max_len, 4);
        }
        const auto t0 = std::chrono::steady_clock::now();
        spoa::Graph graph{};
        for (const auto& read : win.reads) {
          const uint64_t nodes = graph.nodes().size();
          std::int32_t score = 0;
          auto alignment = engine->Align(read, graph, &score);
          my_cells += nodes * read.size();
          if (win.strand) {
            const std::string rc = ReverseComplement(read);
            std::int32_t score_rev = 0;
            auto alignment_rev = engine->Align(rc, graph, &score_rev);
            my_cells += nodes * read.size();
            if (score >= score_rev) {
              graph.AddAlignment(alignment, read);
            } else {
              graph.AddAlignment(alignment_rev, rc);
            }
          } else {
            graph.AddAlignment(alignment, read);
          }
        }
        consensus[w] = graph.GenerateConsensus();
        secs[w] = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      }
    } catch (const std::exception& ex) {
      std::cerr << ex.what() << "\n";
      ++failed;
    }
    cells += my_cells;
  };
  const auto t0 = std::chrono::steady_clock::now();
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t) pool.emplace_back(worker);
  for (auto& t : pool) t.join();
  const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (failed) return 1;
  std::vector<double> sorted = secs;
  std::sort(sorted.begin(), sorted.end());
  auto pct = [&](double f) {
    return sorted.empty() ? 0.0 : sorted[std::min(sorted.size() - 1, (size_t)(f * sorted.size()))];
  };
#if defined(__AVX2__) || defined(__SSE4_1__)
  const char* kind = "simd";
#else
  const char* kind = "sisd";
#endif
  std::printf("{\"windows\": %zu, \"seconds\": %.6f, \"threads\": %d, \"cells\": %llu, "
              "\"window_seconds_p50\": %.6f, \"window_seconds_p99\": %.6f, \"engine\": \"%s\"}\n",
              wins.size(), wall, threads, (unsigned long long)cells.load(), pct(0.50), pct(0.99),
              kind);
  if (argc > 9) {
    std::ofstream out(argv[9]);
    for (const auto& c : consensus) out << c << "\n";
  }
  return 0;
}
