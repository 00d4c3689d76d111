// racecheck_main.cpp - drives the emulated device code over small synthetic
// windows, as a program built with -fsanitize=thread,undefined: the SIMT
// emulation then reports any two threads that touch the same shared or
// global bytes between barriers (one of them writing) and any undefined
// behaviour (signed overflow, bad shifts, misaligned access) of the device
// code.  TEST INFRASTRUCTURE ONLY (tests/test_window_host.py builds and runs
// it).  Built with RACECHECK_MW it drives the W-windows-per-CTA loop, else
// the one-window loop (window_read) with the MSA of the window, the cluster
// form (window_read_cl) and the segmented forward.  Correctness against the oracle is checked by the
// other host tests; this program checks only statuses.
#ifdef RACECHECK_MW
#include "batch_mw_host.cpp"
#else
#include "window_host.cpp"
#endif

#include <cstdio>
#include <string>
#include <vector>

namespace {

struct Rng {
  uint64_t s;
  uint32_t next() {
    s ^= s << 13;
    s ^= s >> 7;
    s ^= s << 17;
    return (uint32_t)(s >> 11);
  }
  uint32_t below(uint32_t n) { return next() % n; }
};

// n reads of a random template of `len` bases, each with about 8 % errors
// (substitutions, insertions, deletions) and some cut short.
std::vector<std::string> window(Rng& rng, uint32_t n, uint32_t len) {
  static const char kBases[] = "ACGT";
  std::string tpl;
  for (uint32_t k = 0; k < len; ++k) tpl += kBases[rng.below(4)];
  std::vector<std::string> reads;
  for (uint32_t r = 0; r < n; ++r) {
    std::string s;
    for (char b : tpl) {
      const uint32_t u = rng.below(100);
      if (u < 3) continue;
      if (u < 6) s += kBases[rng.below(4)];
      s += u < 8 ? kBases[rng.below(4)] : b;
    }
    if (r % 3 == 2) s = s.substr(rng.below((uint32_t)s.size() / 4 + 1));
    reads.push_back(s);
  }
  return reads;
}

struct Flat {
  std::string seqs, quals;
  std::vector<uint64_t> off{0};
  explicit Flat(const std::vector<std::string>& reads) {
    for (const auto& r : reads) {
      seqs += r;
      for (size_t k = 0; k < r.size(); ++k) quals += (char)(33 + (k * 7 + r.size()) % 41);
      off.push_back(seqs.size());
    }
  }
};

const int32_t kGaps[3][4] = {{-8, -8, -8, -8}, {-8, -6, -8, -6}, {-8, -6, -10, -4}};

int failures = 0;

void check(const char* what, int32_t st, int type, int gap) {
  if (st != 0) {
    std::printf("%s: type %d gaps %d: status %d\n", what, type, gap, st);
    ++failures;
  }
}

}  // namespace

int main() {
  Rng rng{0x9E3779B97F4A7C15ull};
#ifdef RACECHECK_MW
  // two and four windows per CTA, every type and gap model, both strands
  for (int W : {2, 4})
    for (int type = 0; type < 3; ++type)
      for (int gap = 0; gap < 3; ++gap) {
        std::vector<std::vector<std::string>> wins;
        for (int w = 0; w < W + 1; ++w) wins.push_back(window(rng, 3, 60 + 20 * w));
        std::vector<std::string> all;
        std::vector<uint32_t> wro{0};
        for (auto& w : wins) {
          all.insert(all.end(), w.begin(), w.end());
          wro.push_back((uint32_t)all.size());
        }
        Flat f(all);
        const uint32_t nw = (uint32_t)wins.size();
        std::vector<int8_t> strands(nw, (int8_t)(gap == 1));
        std::vector<int32_t> scores(all.size()), status(nw, -1);
        std::vector<uint8_t> rev(all.size());
        std::vector<uint64_t> coff{0};
        for (auto& w : wins) coff.push_back(coff.back() + 4 * 200 + 64);
        std::vector<char> cons(coff.back());
        std::vector<uint32_t> clen(nw);
        const int32_t* G = kGaps[gap];
        mw_run(type, 5, -4, G[0], G[1], G[2], G[3], W, nw, wro.data(), f.seqs.data(),
               f.off.data(), strands.data(), scores.data(), rev.data(), cons.data(), coff.data(),
               clen.data(), status.data(), type == 2 ? f.quals.data() : nullptr);
        for (int32_t s : status) check("batch_cta_mw", s, type, gap);
      }
#else
  auto one = [&](const char* what, int type, int gap, int wide, int cpt, uint32_t nt,
                 const std::vector<std::string>& reads, bool strand, bool quals, int cl) {
    Flat f(reads);
    const uint32_t nr = (uint32_t)reads.size();
    std::vector<int32_t> scores(nr), rev(nr);
    const uint64_t cap = 2 * f.seqs.size() + 64 * nr + 64;
    std::vector<int32_t> aln(2 * cap);
    std::vector<uint64_t> aoff(nr + 1);
    std::vector<char> cons(f.seqs.size() + 16);
    uint32_t clen = 0, dims[2] = {0, 0};
    std::vector<char> msa((nr + 1) * (f.seqs.size() + 1));  // rows x at most every base
    const int32_t* G = kGaps[gap];
    const int32_t st =
        cl ? wh_run_cl(type, 5, -4, G[0], G[1], G[2], G[3], cl, nt, nr, f.seqs.data(),
                       f.off.data(), quals ? f.quals.data() : nullptr, strand, scores.data(),
                       rev.data(), aln.data(), cap, aoff.data(), cons.data(),
                       (uint32_t)cons.size(), &clen)
           : wh_run(type, 5, -4, G[0], G[1], G[2], G[3], wide, cpt, nt, nr, f.seqs.data(),
                    f.off.data(), quals ? f.quals.data() : nullptr, strand, scores.data(),
                    rev.data(), aln.data(), cap, aoff.data(), cons.data(),
                    (uint32_t)cons.size(), &clen, msa.data(), msa.size(), dims);
    check(what, st, type, gap);
  };
  // every variant on three (type, gap model) pairs that cover each type and
  // each gap model once; strands and qualities vary with the pair
  for (int v = 0; v < 9; ++v)
    for (int type = 0; type < 3; ++type) {
      const int gap = (3 + v - type) % 3;
      const bool strand = (type + v) % 2 == 1, quals = (gap + v) % 2 == 0;
      switch (v) {
        case 0:  // one warp, 8 columns per thread
          one("window_read 32x8", type, gap, 0, 8, 32, window(rng, 3, 140), strand, quals, 0);
          break;
        case 1:  // the same on the 32-bit width
          one("window_read 32x8 int32", type, gap, 1, 8, 32, window(rng, 3, 140), strand,
              quals, 0);
          break;
        case 2:  // the one-warp build (compile-time tile)
          one("window_read one-warp 32x16", type, gap, 0, 16, 32, window(rng, 3, 280), strand,
              quals, 0);
          break;
        case 3:  // a two-warp CTA (cross-warp scan carries)
          one("window_read 64x8", type, gap, 0, 8, 64, window(rng, 3, 280), strand, quals, 0);
          break;
        case 4:  // the segmented forward: two 12-column strips per thread
          one("window_read segmented", type, gap, 1, -12, 32, window(rng, 3, 450), strand,
              quals, 0);
          break;
        case 8:  // nine warps: the scans' carries across many warps
          one("window_read 288x8", type, gap, 0, 8, 288, window(rng, 2, 300), strand, quals, 0);
          break;
        default:  // clusters of 2, 4 and 8 CTAs (32 threads x 12 columns each)
          one("window_read_cl", type, gap, 1, 12, 32, window(rng, 3, 200), strand, quals,
              v == 5 ? 2 : v == 6 ? 4 : 8);
      }
    }
#endif
  std::printf("%s\n", failures ? "status failures" : "statuses ok");
  return failures ? 1 : 0;
}
