// Stand-in for the few Parthenon / Kokkos names the reference's reconstruction and Riemann
// headers use, so that those headers compile unchanged for a serial CPU build.
//
// TEST INFRASTRUCTURE ONLY: oracle/build_ref.py compiles the reference's own
// src/recon/{dc,plm,ppm}_simple.hpp and src/hydro/rsolvers/hydro_{hlle,hllc,lhllc}.hpp
// against this file (into oracle/_ref/), and tests/test_ref_pin.py checks the oracle's
// restatement against them.  The macro values follow Parthenon's published definitions
// (the oracle's assumption A1).
#ifndef APH_REF_SHIM_PARTHENON_HPP_
#define APH_REF_SHIM_PARTHENON_HPP_

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <limits>
#include <type_traits>

#include "../basic_types.hpp"

#ifndef KOKKOS_INLINE_FUNCTION
#define KOKKOS_INLINE_FUNCTION inline
#endif
#ifndef KOKKOS_FORCEINLINE_FUNCTION
#define KOKKOS_FORCEINLINE_FUNCTION inline
#endif
#define SQR(x) ((x) * (x))
#define SIGN(x) (((x) < 0.0) ? -1.0 : 1.0)
#define TINY_NUMBER 1.0e-20
#define PARTHENON_FAIL(msg)                        \
  {                                                \
    std::fprintf(stderr, "reference shim: %s\n", msg); \
    std::abort();                                  \
  }

namespace parthenon {

constexpr int X1DIR = 1, X2DIR = 2, X3DIR = 3;

// One team of one thread: inner loops run serially in index order.
struct team_mbr_t {
  void team_barrier() const {}
};

template <class F>
inline void par_for_inner(const team_mbr_t &, int il, int iu, F &&f) {
  for (int i = il; i <= iu; ++i) f(i);
}

// (n, i) scratch array over caller-owned storage; element access returns a reference
// through a const view, as Kokkos views do.
template <class T>
struct ScratchPad2D {
  T *data = nullptr;
  int n1 = 0;  // extent of i
  ScratchPad2D() = default;
  ScratchPad2D(T *d, int /*nvar*/, int ni) : data(d), n1(ni) {}
  T &operator()(int n, int i) const { return data[(long)n * n1 + i]; }
};

// (n, k, j, i) field of one block, i fastest.
template <class T>
struct VariablePack {
  T *data = nullptr;
  int dim[5] = {0, 0, 0, 0, 0};  // dim[1] = ni, dim[2] = nj, dim[3] = nk, dim[4] = nvar
  VariablePack() = default;
  VariablePack(T *d, int nvar, int nk, int nj, int ni) : data(d) {
    dim[1] = ni;
    dim[2] = nj;
    dim[3] = nk;
    dim[4] = nvar;
  }
  int GetDim(int d) const { return dim[d]; }
  T &operator()(int n, int k, int j, int i) const {
    return data[(((long)n * dim[3] + k) * dim[2] + j) * dim[1] + i];
  }
};

// A block's conserved field with one face-flux array per direction, each shaped like the field.
template <class T>
struct VariableFluxPack : VariablePack<T> {
  T *fx[3] = {nullptr, nullptr, nullptr};
  using VariablePack<T>::dim;
  T &flux(int dir, int n, int k, int j, int i) const {
    return fx[dir - 1][(((long)n * dim[3] + k) * dim[2] + j) * dim[1] + i];
  }
};

template <class T>
using ParArray4D = VariablePack<T>;

}  // namespace parthenon

#endif  // APH_REF_SHIM_PARTHENON_HPP_
