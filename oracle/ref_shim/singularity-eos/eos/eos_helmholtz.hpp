// Stand-in for a singularity-eos header (test infrastructure): the reference's Riemann
// solvers take an EOS argument they do not use, so empty types suffice.
#include "eos_variant.hpp"
