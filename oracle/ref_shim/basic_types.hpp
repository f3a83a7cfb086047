// Stand-in for Parthenon's basic_types.hpp (test infrastructure; see parthenon/parthenon.hpp).
#ifndef APH_REF_SHIM_BASIC_TYPES_HPP_
#define APH_REF_SHIM_BASIC_TYPES_HPP_
#include <limits>
namespace parthenon {
using Real = double;
}
#endif
