// spoa/spoa.hpp - umbrella header, as in spoa v4 (include/spoa/spoa.hpp).
#ifndef SPOA_SPOA_HPP_
#define SPOA_SPOA_HPP_

#include "spoa/alignment_engine.hpp"
#include "spoa/graph.hpp"

#endif  // SPOA_SPOA_HPP_
