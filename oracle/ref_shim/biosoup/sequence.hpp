// biosoup/sequence.hpp - stand-in for biosoup 0.10.0's Sequence, the one
// type of that library the reference CLI (src/main.cpp) uses.
//
// TEST INFRASTRUCTURE ONLY: lets oracle/Makefile compile the reference's
// own, unmodified src/main.cpp into oracle/_ref/spoa_ref_cli (biosoup is
// fetched by the reference's CMake build and is not part of its tree).
// Restated from biosoup's published interface: a named sequence with
// optional quality; ReverseAndComplement pairs Watson-Crick and IUPAC
// codes, reverses the data and reverses the quality.
#ifndef ORACLE_SHIM_BIOSOUP_SEQUENCE_HPP_
#define ORACLE_SHIM_BIOSOUP_SEQUENCE_HPP_

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <string>

namespace biosoup {

struct Sequence {
  Sequence() = default;
  Sequence(const char* name, std::uint32_t name_len, const char* data,
           std::uint32_t data_len)
      : id(num_objects++), name(name, name_len), data(data, data_len) {}
  Sequence(const char* name, std::uint32_t name_len, const char* data,
           std::uint32_t data_len, const char* quality, std::uint32_t quality_len)
      : id(num_objects++),
        name(name, name_len),
        data(data, data_len),
        quality(quality, quality_len) {}

  void ReverseAndComplement() {
    for (auto& ch : data) ch = Complement(ch);
    std::reverse(data.begin(), data.end());
    std::reverse(quality.begin(), quality.end());
  }

  static char Complement(char ch) {
    switch (ch) {
      case 'A': return 'T'; case 'C': return 'G'; case 'G': return 'C';
      case 'T': return 'A'; case 'U': return 'A'; case 'R': return 'Y';
      case 'Y': return 'R'; case 'K': return 'M'; case 'M': return 'K';
      case 'B': return 'V'; case 'D': return 'H'; case 'H': return 'D';
      case 'V': return 'B'; case 'a': return 't'; case 'c': return 'g';
      case 'g': return 'c'; case 't': return 'a'; case 'u': return 'a';
      default: return ch;
    }
  }

  static std::atomic<std::uint32_t> num_objects;

  std::uint32_t id = 0;
  std::string name;
  std::string data;
  std::string quality;
};

}  // namespace biosoup

#endif  // ORACLE_SHIM_BIOSOUP_SEQUENCE_HPP_
