// gfa_host.cpp - the GFA writer of the C ABI (spoa_gb300/csrc/gfa_text.h)
// on exported arrays, for the CPU test suite (tests/test_gfa_text.py
// compares it with the oracle's GFA, which matches the reference's).
// TEST INFRASTRUCTURE ONLY.
#include <cstring>

#include "../../spoa_gb300/csrc/gfa_text.h"

extern "C" uint64_t gh_gfa(uint32_t n_nodes, uint32_t n_seqs, uint32_t n_consensus,
                           const uint8_t* chars, const uint32_t* out_off,
                           const uint32_t* out_edges, const uint32_t* e_head,
                           const int64_t* e_weight, const uint32_t* label_off,
                           const uint32_t* labels, const uint32_t* seq_begin,
                           const uint32_t* consensus, const char* const* headers,
                           const uint8_t* is_reversed, int32_t include_consensus, char* out,
                           uint64_t cap) {
  spoa_gb300::GfaGraph g{n_nodes, n_seqs,  n_consensus, chars,     out_off,  out_edges,
                         e_head,  e_weight, label_off,  labels,    seq_begin, consensus};
  const std::string s = spoa_gb300::gfa_text(g, headers, is_reversed, include_consensus != 0);
  if (s.size() <= cap) std::memcpy(out, s.data(), s.size());
  return s.size();
}
