// aph_amr.cuh -- ghost cells and flux correction on a statically refined 2D mesh.
//
// Shared by the per-pack kernels and the batched stage kernel.  Ghost cells across a face
// are computed from the neighbours' interiors only (so one pass fills every block):
//   same level    copy of the neighbour's cell;
//   finer         mean of the 2x2 fine cells, ((a+b)+(c+d))*0.25;
//   coarser       minmod-limited linear prolongation c + o_n s_n + o_t s_t, o = -/+ 1/4 by the
//                 fine cell's parity; the normal slope takes its fine-side neighbour as the
//                 restricted mean of this block's own edge cells; the transverse slope uses
//                 the coarse block's interior neighbours and is 0 at its edge;
//   boundary      outflow copy / reflecting mirror with the normal momentum negated;
// (every component alike, passive scalars included)
//   corner ghosts copy the nearest interior cell (no flux pass reads them).
// Every product in these formulas is by a power of two, so fused and unfused arithmetic
// round identically.
#pragma once
#include "aph_internal.h"
#include "aph_math.cuh"

namespace aph {

template <class BLK>
__device__ __forceinline__ long long amr_cell(const BLK &B, int ng, int d, int a, int t) {
  const int i = d == 0 ? ng + a : ng + t;
  const int j = d == 0 ? ng + t : ng + a;
  return (long long)j * B.ni + i;
}

__device__ __forceinline__ double amr_minmod(double a, double b) {
  if (!is_pos(a * b)) return 0.0;
  return mag(a) < mag(b) ? a : b;
}

// The finer neighbour of face `face` of B that covers fine transverse global index tg2.
template <class BLK>
__device__ __forceinline__ const BLK &amr_fine_nbr(const BLK *blocks, const BLK &B, int face,
                                                   int td, int tg2) {
  int pick = B.amr.nbr[face][0];
  for (int n = 0; n < B.amr.cnt[face]; ++n) {
    const BLK &C = blocks[B.amr.nbr[face][n]];
    if (tg2 >= C.amr.origin[td] && tg2 < C.amr.origin[td] + C.nx[td]) pick = B.amr.nbr[face][n];
  }
  return blocks[pick];
}

// Ghost value of component v across face (d, s) of block B at depth k, transverse index t,
// for the state q(block, component, cell).
template <class BLK, class Q>
__device__ double amr_ghost(const BLK *blocks, const BLK &B, Q q, const int (*bc)[2], int ng, int d,
                            int s, int k, int t, int v) {
  const int face = 2 * d + s, td = 1 - d;
  const int kind = B.amr.kind[face];
  if (kind == FACE_SAME) {
    const BLK &N = blocks[B.amr.nbr[face][0]];
    const int a = s == 0 ? N.nx[d] - 1 - k : k;
    const int tn = B.amr.origin[td] + t - N.amr.origin[td];
    return q(N, v, amr_cell(N, ng, d, a, tn));
  }
  if (kind == FACE_BOUNDARY) {
    if (bc[d][s] == 1) return q(B, v, amr_cell(B, ng, d, s == 0 ? 0 : B.nx[d] - 1, t));  // outflow
    const double x = q(B, v, amr_cell(B, ng, d, s == 0 ? k : B.nx[d] - 1 - k, t));      // reflecting
    return (v == 1 + d) ? -x : x;
  }
  if (kind == FACE_FINER) {
    const int tg2 = 2 * (B.amr.origin[td] + t);
    const BLK &F = amr_fine_nbr(blocks, B, face, td, tg2);
    const int ft = tg2 - F.amr.origin[td];
    const int a0 = s == 0 ? F.nx[d] - 1 - 2 * k : 2 * k;
    const int a1 = s == 0 ? a0 - 1 : a0 + 1;
    return ((q(F, v, amr_cell(F, ng, d, a0, ft)) + q(F, v, amr_cell(F, ng, d, a0, ft + 1))) +
            (q(F, v, amr_cell(F, ng, d, a1, ft)) + q(F, v, amr_cell(F, ng, d, a1, ft + 1)))) *
           0.25;
  }
  // coarser neighbour: prolongation
  const BLK &C = blocks[B.amr.nbr[face][0]];
  const int tg = B.amr.origin[td] + t;
  const int tc = (tg >> 1) - C.amr.origin[td];
  const int kc = k >> 1;
  const int ic = s == 0 ? C.nx[d] - 1 - kc : kc;
  const int gf = s == 0 ? B.amr.origin[d] - 1 - k : B.amr.origin[d] + B.nx[d] + k;
  const double on = (gf & 1) ? 0.25 : -0.25;
  const double ot = (tg & 1) ? 0.25 : -0.25;
  const int tf0 = 2 * (tc + C.amr.origin[td]) - B.amr.origin[td];
  const bool has_t = tc - 1 >= 0 && tc + 1 < C.nx[td];
  auto pc = [&](int a, int tt) { return q(C, v, amr_cell(C, ng, d, a, tt)); };
  auto pb = [&](int a, int tt) { return q(B, v, amr_cell(B, ng, d, a, tt)); };
  const double c = pc(ic, tc);
  auto restricted = [&](int a0, int a1) {
    return ((pb(a0, tf0) + pb(a0, tf0 + 1)) + (pb(a1, tf0) + pb(a1, tf0 + 1))) * 0.25;
  };
  double cm, cp;
  if (s == 0) {
    cm = pc(ic - 1, tc);
    cp = ic + 1 < C.nx[d] ? pc(ic + 1, tc) : restricted(0, 1);
  } else {
    cm = ic - 1 >= 0 ? pc(ic - 1, tc) : restricted(B.nx[d] - 1, B.nx[d] - 2);
    cp = pc(ic + 1, tc);
  }
  const double sn = amr_minmod(c - cm, cp - c);
  double st = 0.0;
  if (has_t) st = amr_minmod(c - pc(ic, tc - 1), pc(ic, tc + 1) - c);
  return c + on * sn + ot * st;
}

// Fill the ghost cell c (entire-domain index) of block B's field dst (nvar x ncell) from
// the state q(block, component, cell).
template <class BLK, class Q>
__device__ void amr_fill_cell(const BLK *blocks, const BLK &B, Q q, double *dst, int nvar,
                              const int (*bc)[2], int ng, long long c) {
  const int i = (int)(c % B.ni), j = (int)(c / B.ni);
  const bool gi = i < ng || i >= ng + B.nx[0];
  const bool gj = j < ng || j >= ng + B.nx[1];
  if (!gi && !gj) return;
  if (gi && gj) {
    const int ci = min(max(i, ng), ng + B.nx[0] - 1);
    const int cj = min(max(j, ng), ng + B.nx[1] - 1);
    for (int v = 0; v < nvar; ++v) dst[v * B.ncell + c] = q(B, v, (long long)cj * B.ni + ci);
  } else if (gi) {
    const int s = i < ng ? 0 : 1;
    const int k = s == 0 ? ng - 1 - i : i - (ng + B.nx[0]);
    for (int v = 0; v < nvar; ++v) dst[v * B.ncell + c] = amr_ghost(blocks, B, q, bc, ng, 0, s, k, j - ng, v);
  } else {
    const int s = j < ng ? 0 : 1;
    const int k = s == 0 ? ng - 1 - j : j - (ng + B.nx[1]);
    for (int v = 0; v < nvar; ++v) dst[v * B.ncell + c] = amr_ghost(blocks, B, q, bc, ng, 1, s, k, i - ng, v);
  }
}

}  // namespace aph
