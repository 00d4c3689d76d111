// cereal/types/utility.hpp - see cereal/access.hpp (test infrastructure only).
#include "cereal/access.hpp"
