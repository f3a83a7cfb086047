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

// Where the ghost cell (d, s, k, t) of block B takes its values from: the neighbour blocks and
// cells of its kind, resolved once for all components.
template <class BLK>
struct GhostSrc {
  int kind;                    // FACE_SAME, FACE_BOUNDARY (outflow / reflect), FACE_FINER, FACE_COARSER
  int flip;                    // reflecting: the component negated (1 + d), else -1
  const BLK *X;                // SAME / BOUNDARY: the source block; FINER: the fine block; COARSER: C
  long long c0, c1, c2, c3;    // SAME / BOUNDARY: c0; FINER: the 2x2 fine cells;
                               // COARSER: c0 the parent, c1 / c2 its normal neighbours (-1: restricted
                               // from B's own edge cells r0..r3), c3 unused
  long long t0, t1;            // COARSER: transverse neighbours (-1: no transverse slope)
  long long r0, r1, r2, r3;    // COARSER: B's 2x2 edge cells for a restricted normal neighbour
  double on, ot;
};

template <class BLK>
__device__ GhostSrc<BLK> amr_ghost_src(const BLK *blocks, const BLK &B, const int (*bc)[2], int ng, int d,
                                       int s, int k, int t) {
  GhostSrc<BLK> g;
  const int face = 2 * d + s, td = 1 - d;
  g.kind = B.amr.kind[face];
  g.flip = -1;
  g.c1 = g.c2 = g.c3 = g.t0 = g.t1 = g.r0 = g.r1 = g.r2 = g.r3 = -1;
  g.on = g.ot = 0.0;
  if (g.kind == FACE_SAME) {
    const BLK &N = blocks[B.amr.nbr[face][0]];
    g.X = &N;
    g.c0 = amr_cell(N, ng, d, s == 0 ? N.nx[d] - 1 - k : k, B.amr.origin[td] + t - N.amr.origin[td]);
  } else if (g.kind == FACE_BOUNDARY) {
    g.X = &B;
    if (bc[d][s] == 1) {  // outflow
      g.c0 = amr_cell(B, ng, d, s == 0 ? 0 : B.nx[d] - 1, t);
    } else {              // reflecting
      g.c0 = amr_cell(B, ng, d, s == 0 ? k : B.nx[d] - 1 - k, t);
      g.flip = 1 + d;
    }
  } else if (g.kind == FACE_FINER) {
    const int tg2 = 2 * (B.amr.origin[td] + t);
    const BLK &F = amr_fine_nbr(blocks, B, face, td, tg2);
    const int ft = tg2 - F.amr.origin[td];
    const int a0 = s == 0 ? F.nx[d] - 1 - 2 * k : 2 * k;
    const int a1 = s == 0 ? a0 - 1 : a0 + 1;
    g.X = &F;
    g.c0 = amr_cell(F, ng, d, a0, ft);
    g.c1 = amr_cell(F, ng, d, a0, ft + 1);
    g.c2 = amr_cell(F, ng, d, a1, ft);
    g.c3 = amr_cell(F, ng, d, a1, ft + 1);
  } else {  // coarser neighbour: prolongation
    const BLK &C = blocks[B.amr.nbr[face][0]];
    const int tg = B.amr.origin[td] + t;
    const int tc = (tg >> 1) - C.amr.origin[td];
    const int kc = k >> 1;
    const int ic = s == 0 ? C.nx[d] - 1 - kc : kc;
    const int gf = s == 0 ? B.amr.origin[d] - 1 - k : B.amr.origin[d] + B.nx[d] + k;
    g.on = (gf & 1) ? 0.25 : -0.25;
    g.ot = (tg & 1) ? 0.25 : -0.25;
    g.X = &C;
    g.c0 = amr_cell(C, ng, d, ic, tc);
    const int tf0 = 2 * (tc + C.amr.origin[td]) - B.amr.origin[td];
    bool restricted = false;
    int ra0 = 0, ra1 = 0;
    if (s == 0) {
      g.c1 = amr_cell(C, ng, d, ic - 1, tc);
      if (ic + 1 < C.nx[d]) g.c2 = amr_cell(C, ng, d, ic + 1, tc);
      else { restricted = true; ra0 = 0; ra1 = 1; }
    } else {
      if (ic - 1 >= 0) g.c1 = amr_cell(C, ng, d, ic - 1, tc);
      else { restricted = true; ra0 = B.nx[d] - 1; ra1 = B.nx[d] - 2; }
      g.c2 = amr_cell(C, ng, d, ic + 1, tc);
    }
    if (restricted) {
      g.r0 = amr_cell(B, ng, d, ra0, tf0);
      g.r1 = amr_cell(B, ng, d, ra0, tf0 + 1);
      g.r2 = amr_cell(B, ng, d, ra1, tf0);
      g.r3 = amr_cell(B, ng, d, ra1, tf0 + 1);
    }
    if (tc - 1 >= 0 && tc + 1 < C.nx[td]) {
      g.t0 = amr_cell(C, ng, d, ic, tc - 1);
      g.t1 = amr_cell(C, ng, d, ic, tc + 1);
    }
  }
  return g;
}

// Ghost value of component v from its sources, for the state q(block, component, cell).
template <class BLK, class Q>
__device__ __forceinline__ double amr_ghost_value(const GhostSrc<BLK> &g, const BLK &B, Q q, int v) {
  if (g.kind == FACE_SAME) return q(*g.X, v, g.c0);
  if (g.kind == FACE_BOUNDARY) {
    const double x = q(*g.X, v, g.c0);
    return v == g.flip ? -x : x;
  }
  if (g.kind == FACE_FINER)
    return ((q(*g.X, v, g.c0) + q(*g.X, v, g.c1)) + (q(*g.X, v, g.c2) + q(*g.X, v, g.c3))) * 0.25;
  const BLK &C = *g.X;
  const double c = q(C, v, g.c0);
  double cm, cp;
  if (g.r0 >= 0) {
    const double r = ((q(B, v, g.r0) + q(B, v, g.r1)) + (q(B, v, g.r2) + q(B, v, g.r3))) * 0.25;
    cm = g.c1 >= 0 ? q(C, v, g.c1) : r;
    cp = g.c2 >= 0 ? q(C, v, g.c2) : r;
  } else {
    cm = q(C, v, g.c1);
    cp = q(C, v, g.c2);
  }
  const double sn = amr_minmod(c - cm, cp - c);
  double st = 0.0;
  if (g.t0 >= 0) st = amr_minmod(c - q(C, v, g.t0), q(C, v, g.t1) - c);
  return c + g.on * sn + g.ot * st;
}

// The five hydro components of the ghost cell (d, s, k, t) of block B in one pass over its
// sources (packs without passive scalars), for the state q(block, component, cell).
template <class BLK, class Q>
__device__ void amr_ghost5(const BLK *blocks, const BLK &B, Q q, const int (*bc)[2], int ng,
                          int d, int s, int k, int t, double *out) {
  const int face = 2 * d + s, td = 1 - d;
  const int kind = B.amr.kind[face];
  if (kind == FACE_SAME) {
    const BLK &N = blocks[B.amr.nbr[face][0]];
    const int a = s == 0 ? N.nx[d] - 1 - k : k;
    const int tn = B.amr.origin[td] + t - N.amr.origin[td];
    const long long c = amr_cell(N, ng, d, a, tn);
#pragma unroll
    for (int v = 0; v < NHYDRO; ++v) out[v] = q(N, v, c);
  } else if (kind == FACE_BOUNDARY) {
    if (bc[d][s] == 1) {  // outflow
      const long long c = amr_cell(B, ng, d, s == 0 ? 0 : B.nx[d] - 1, t);
#pragma unroll
      for (int v = 0; v < NHYDRO; ++v) out[v] = q(B, v, c);
    } else {              // reflecting
      const long long c = amr_cell(B, ng, d, s == 0 ? k : B.nx[d] - 1 - k, t);
#pragma unroll
      for (int v = 0; v < NHYDRO; ++v) {
        const double x = q(B, v, c);
        out[v] = (v == 1 + d) ? -x : x;
      }
    }
  } else if (kind == FACE_FINER) {
    const int tg2 = 2 * (B.amr.origin[td] + t);
    const BLK &F = amr_fine_nbr(blocks, B, face, td, tg2);
    const int ft = tg2 - F.amr.origin[td];
    const int a0 = s == 0 ? F.nx[d] - 1 - 2 * k : 2 * k;
    const int a1 = s == 0 ? a0 - 1 : a0 + 1;
    const long long c00 = amr_cell(F, ng, d, a0, ft), c01 = amr_cell(F, ng, d, a0, ft + 1);
    const long long c10 = amr_cell(F, ng, d, a1, ft), c11 = amr_cell(F, ng, d, a1, ft + 1);
#pragma unroll
    for (int v = 0; v < NHYDRO; ++v)
      out[v] = ((q(F, v, c00) + q(F, v, c01)) + (q(F, v, c10) + q(F, v, c11))) * 0.25;
  } else {  // coarser neighbour: prolongation
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
#pragma unroll
    for (int v = 0; v < NHYDRO; ++v) {
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
      out[v] = c + on * sn + ot * st;
    }
  }
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
    return;
  }
  const int d = gi ? 0 : 1;
  const int s = gi ? (i < ng ? 0 : 1) : (j < ng ? 0 : 1);
  const int k = gi ? (s == 0 ? ng - 1 - i : i - (ng + B.nx[0])) : (s == 0 ? ng - 1 - j : j - (ng + B.nx[1]));
  const int t = gi ? j - ng : i - ng;
  if (nvar == NHYDRO) {
    double val[NHYDRO];
    amr_ghost5(blocks, B, q, bc, ng, d, s, k, t, val);
#pragma unroll
    for (int v = 0; v < NHYDRO; ++v) dst[v * B.ncell + c] = val[v];
    return;
  }
  const GhostSrc<BLK> g = amr_ghost_src(blocks, B, bc, ng, d, s, k, t);
  for (int v = 0; v < nvar; ++v) dst[v * B.ncell + c] = amr_ghost_value(g, B, q, v);
}

}  // namespace aph
