// spoa/alignment_engine.hpp - spoa's AlignmentEngine interface, backed by the
// GB300 library (libspoa.so over libspoa_gb300.so).
//
// Source-compatible with spoa v4's include/spoa/alignment_engine.hpp: the
// same namespace, enums, factory overloads and virtual interface, so spoa's
// callers (src/main.cpp:252-314, test/spoa_test.cpp, polishers) compile
// against it unchanged.  Create returns a CudaAlignmentEngine, whose Align
// runs the graph-to-sequence DP and its traceback on the GPU.
#ifndef SPOA_ALIGNMENT_ENGINE_HPP_
#define SPOA_ALIGNMENT_ENGINE_HPP_

#include <cstdint>
#include <memory>
#include <string>
#include <utility>
#include <vector>

namespace spoa {

// include/spoa/alignment_engine.hpp:16-26 of the reference
enum class AlignmentType {
  kSW,  // local (Smith-Waterman)
  kNW,  // global (Needleman-Wunsch)
  kOV   // overlap
};

enum class AlignmentSubtype {
  kLinear,  // g * i
  kAffine,  // g + (i - 1) * e
  kConvex   // the better of two affine gap costs
};

class Graph;

// (node id or -1, sequence position or -1) per aligned column
using Alignment = std::vector<std::pair<std::int32_t, std::int32_t>>;

class AlignmentEngine {
 public:
  virtual ~AlignmentEngine() = default;

  // The three factory overloads of the reference (alignment_engine.cpp:15-73):
  // validation, gap-model resolution and canonical penalties.  Throws
  // std::invalid_argument with the reference's messages.
  static std::unique_ptr<AlignmentEngine> Create(
      AlignmentType type, std::int8_t m, std::int8_t n, std::int8_t g);

  static std::unique_ptr<AlignmentEngine> Create(
      AlignmentType type, std::int8_t m, std::int8_t n, std::int8_t g, std::int8_t e);

  static std::unique_ptr<AlignmentEngine> Create(
      AlignmentType type, std::int8_t m, std::int8_t n, std::int8_t g, std::int8_t e,
      std::int8_t q, std::int8_t c);

  virtual void Prealloc(std::uint32_t max_sequence_len, std::uint8_t alphabet_size) = 0;

  Alignment Align(const std::string& sequence, const Graph& graph,
                  std::int32_t* score = nullptr);

  virtual Alignment Align(const char* sequence, std::uint32_t sequence_len,
                          const Graph& graph, std::int32_t* score = nullptr) = 0;

  AlignmentType type() const { return type_; }
  AlignmentSubtype subtype() const { return subtype_; }

 protected:
  AlignmentEngine(AlignmentType type, AlignmentSubtype subtype, std::int8_t m, std::int8_t n,
                  std::int8_t g, std::int8_t e, std::int8_t q, std::int8_t c);

  // alignment_engine.cpp:101-110
  std::int64_t WorstCaseAlignmentScore(std::int64_t sequence_len, std::int64_t graph_len) const;

  AlignmentType type_;
  AlignmentSubtype subtype_;
  std::int8_t m_;
  std::int8_t n_;
  std::int8_t g_;
  std::int8_t e_;
  std::int8_t q_;
  std::int8_t c_;
};

}  // namespace spoa

#endif  // SPOA_ALIGNMENT_ENGINE_HPP_
