// Stand-in for singularity-eos's variant header (test infrastructure): the reference's
// Riemann solvers take an EOS argument they do not use, so empty types suffice.
#ifndef APH_REF_SHIM_EOS_VARIANT_HPP_
#define APH_REF_SHIM_EOS_VARIANT_HPP_
namespace singularity {
struct IdealGas {};
struct Helmholtz {};
template <class... Ts>
struct Variant {};
}  // namespace singularity
#endif
