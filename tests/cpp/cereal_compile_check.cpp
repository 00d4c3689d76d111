// cereal_compile_check.cpp - a spoa caller that persists its graph through
// cereal (`archive(graph)`, as with the reference's SPOA_USE_CEREAL build)
// compiles against include/spoa/graph.hpp unchanged.  Compiled, not run,
// by tests/test_cpp_api.py, with the archive stand-ins of the oracle.
#include <string>

#include "cereal/access.hpp"
#include "spoa/spoa.hpp"

void Persist(const spoa::Graph& graph, std::string* bytes) {
  cereal::BinaryOutputArchive out(bytes);
  out(graph);
}

void Restore(const std::string& bytes, spoa::Graph* graph) {
  cereal::BinaryInputArchive in(bytes);
  in(*graph);
}
