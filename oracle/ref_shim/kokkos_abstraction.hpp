// Stand-in for Parthenon's kokkos_abstraction.hpp (test infrastructure; see parthenon/parthenon.hpp).
#include "parthenon/parthenon.hpp"
