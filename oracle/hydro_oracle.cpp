// hydro_oracle.cpp -- CPU FP64 restatement of apophis's hydro flux path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: the tests, the smoke
// check and the CPU-baseline leg of the benchmark load it to check (or time beside)
// the CUDA path.  Nothing in the product links or calls it.
//
// Every function below restates one piece of the reference, in the reference's
// operation order, so that a build with -O2 -ffp-contract=off reproduces the
// reference's own FP64 CPU arithmetic (no FMA contraction):
//   ConsToPrim<IdealGas>        src/hydro/hydro.cpp:422-533
//   EstimateTimestep<euler>     src/hydro/hydro.cpp:351-420
//   CalculateFluxes<...>        src/hydro/hydro.cpp:535-744 (index ranges included)
//   DC / PLM / PPM              src/recon/dc_simple.hpp, plm_simple.hpp, ppm_simple.hpp
//   HLLE / HLLC / LHLLC / none  src/hydro/rsolvers/hydro_{hlle,hllc,lhllc,none}.hpp
//   stage order of one RK step  src/apophis_driver.cpp:27-129
//   reflecting boundaries       src/boundaries/apophis_boundaries.cpp:18-92
//   constant-g source           src/gravity/gravity.cpp:374-410
//
// Semantics that live in un-vendored dependencies (Parthenon, singularity-eos; the
// submodules are empty and carry no pinned commit) are restated from their published
// behaviour and collected in the ASSUMPTIONS block right below.  Parity of those
// pieces against the true reference binary is unpinned: the reference cannot be
// built here.
//
// ASSUMPTIONS (Parthenon / singularity-eos):
//  A1 SQR(x) = x*x; SIGN(x) = (x < 0) ? -1 : 1; TINY_NUMBER = 1e-20   (parthenon defs)
//  A2 IdealGas(gm1, cv): P(rho,e) = max(0, gm1*rho*e);
//     B(rho,e) = max(10*DBL_MIN, gm1*(gm1+1)*rho*e)                     (singularity-eos)
//  A3 UpdateWithFluxDivergence: u0 = gam0*u0 + gam1*u1 + beta_dt*FluxDivergence,
//     FluxDivergence = -du/V with du = sum_d (A_d*F_d(+) - A_d*F_d(-)),
//     uniform Cartesian A_1 = dx2*dx3, A_2 = dx1*dx3, A_3 = dx1*dx2, V = dx1*dx2*dx3
//  A4 low-storage RK coefficients (gam0, gam1, beta) per stage:
//     rk1 (0,1,1); rk2 (0,1,1),(1/2,1/2,1/2); rk3 (0,1,1),(1/4,3/4,1/4),(2/3,1/3,2/3);
//     vl2 (0,1,1/2),(0,1,1); vl2's first stage uses donor-cell reconstruction
//     (src/hydro/hydro.cpp:128-131)
//  A5 dt policy: dt_0 = EstimateTimestep(U^0); dt_n = min(2*dt_{n-1}, EstimateTimestep(U^n));
//     dt is clipped so that t never passes tlim
//  A6 ghost zones: same-level exchange then physical boundaries; ghost cell values are a
//     per-dimension map of the global cell index (periodic wrap, outflow clamp,
//     reflect mirror with the normal momentum negated)
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

typedef double Real;

// Variable indices: src/main.hpp:6-20
enum { IDN = 0, IM1 = 1, IM2 = 2, IM3 = 3, IEN = 4, NHYDRO = 5 };
enum { IV1 = 1, IV2 = 2, IV3 = 3, IPR = 4 };
// Enumerations: src/main.hpp:32-53
enum { RECON_DC = 1, RECON_PLM = 2, RECON_PPM = 3 };
enum { RS_NONE = 1, RS_HLLE = 2, RS_HLLC = 3, RS_LHLLC = 4 };
enum { INT_RK1 = 1, INT_RK2 = 2, INT_RK3 = 3, INT_VL2 = 4 };
enum { BC_PERIODIC = 0, BC_OUTFLOW = 1, BC_REFLECT = 2 };

static const Real C_LIGHT = 2.99792458e10;   // hydro_hlle.hpp:26, hydro.cpp:353
static const Real TINY_NUMBER = 1.0e-20;      // A1

static inline Real SQR(Real x) { return x * x; }
static inline Real SIGN(Real x) { return (x < 0.0) ? -1.0 : 1.0; }
// std::min / std::max semantics (first argument wins ties)
static inline Real smin(Real a, Real b) { return (b < a) ? b : a; }
static inline Real smax(Real a, Real b) { return (a < b) ? b : a; }

// ---- IdealGas (A2) ----------------------------------------------------------
static inline Real eos_pressure(Real gm1, Real rho, Real sie) {
  Real p = gm1 * rho * sie;
  return (0.0 > p) ? 0.0 : p;
}
static inline Real eos_bulk_modulus(Real gm1, Real rho, Real sie) {
  const Real small = 10.0 * DBL_MIN;
  Real b = gm1 * (gm1 + 1.0) * rho * sie;
  return (small < b) ? b : small;
}

struct Dims {
  int nvar, ni, nj, nk;  // entire-domain extents (ghosts included)
  int nx1, nx2, nx3, ng, ndim;
  int is, ie, js, je, ks, ke;
  size_t ncell;
};

static Dims make_dims(int nvar, int nx1, int nx2, int nx3, int ng, int ndim) {
  Dims d;
  d.nvar = nvar; d.nx1 = nx1; d.nx2 = nx2; d.nx3 = nx3; d.ng = ng; d.ndim = ndim;
  d.ni = nx1 + 2 * ng;
  d.nj = (ndim >= 2) ? nx2 + 2 * ng : 1;
  d.nk = (ndim >= 3) ? nx3 + 2 * ng : 1;
  d.is = ng; d.ie = ng + nx1 - 1;
  d.js = (ndim >= 2) ? ng : 0; d.je = (ndim >= 2) ? ng + nx2 - 1 : 0;
  d.ks = (ndim >= 3) ? ng : 0; d.ke = (ndim >= 3) ? ng + nx3 - 1 : 0;
  d.ncell = (size_t)d.ni * d.nj * d.nk;
  return d;
}

static inline size_t IX(const Dims &d, int n, int k, int j, int i) {
  return (((size_t)n * d.nk + k) * d.nj + j) * d.ni + i;
}

// ---- ConsToPrim: src/hydro/hydro.cpp:422-533 (ideal gas, update_lambda=false) ----
static void cons_to_prim(const Dims &d, Real *cons, Real *prim, Real *gamma, Real gm1,
                         Real dfloor, Real pfloor) {
  const int nscalars = d.nvar - NHYDRO;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < d.nk; ++k)
    for (int j = 0; j < d.nj; ++j)
      for (int i = 0; i < d.ni; ++i) {
        Real &u_d = cons[IX(d, IDN, k, j, i)];
        Real &u_m1 = cons[IX(d, IM1, k, j, i)];
        Real &u_m2 = cons[IX(d, IM2, k, j, i)];
        Real &u_m3 = cons[IX(d, IM3, k, j, i)];
        Real &u_e = cons[IX(d, IEN, k, j, i)];
        Real &w_d = prim[IX(d, IDN, k, j, i)];
        Real &w_vx = prim[IX(d, IV1, k, j, i)];
        Real &w_vy = prim[IX(d, IV2, k, j, i)];
        Real &w_vz = prim[IX(d, IV3, k, j, i)];
        Real &w_p = prim[IX(d, IPR, k, j, i)];
        // apply density floor, without changing momentum or energy (hydro.cpp:475)
        u_d = (u_d > dfloor) ? u_d : dfloor;
        w_d = u_d;
        Real di = 1.0 / u_d;
        w_vx = u_m1 * di;
        w_vy = u_m2 * di;
        w_vz = u_m3 * di;
        Real e_k = 0.5 * di * (SQR(u_m1) + SQR(u_m2) + SQR(u_m3));
        w_p = eos_pressure(gm1, u_d, (u_e - e_k) / u_d);
        Real gm1q = w_p / (u_d * e_k);  // hydro.cpp:517 (kinetic, not internal, energy)
        // apply pressure floor, correct total energy (hydro.cpp:520-521)
        u_e = (w_p > pfloor) ? u_e : ((pfloor / gm1q) + e_k);
        w_p = (w_p > pfloor) ? w_p : pfloor;
        Real g_c = eos_bulk_modulus(gm1, u_d, (u_e - e_k) / u_d) / w_p;
        Real g_e = w_p / (u_e - e_k) + 1;
        if (gamma) {
          gamma[IX(d, 0, k, j, i)] = g_c;
          gamma[IX(d, 1, k, j, i)] = g_e;
        }
        for (int n = NHYDRO; n < NHYDRO + nscalars; ++n)
          prim[IX(d, n, k, j, i)] = cons[IX(d, n, k, j, i)] * di;
      }
}

// ---- Reconstruction: src/recon/*.hpp -----------------------------------------
static inline void PLM(Real q_im1, Real q_i, Real q_ip1, Real &ql_ip1, Real &qr_i) {
  Real dql = (q_i - q_im1);
  Real dqr = (q_ip1 - q_i);
  Real dq2 = dql * dqr;
  Real dqm = 0.0;
  if (dq2 > 0.0) dqm = dq2 / (dql + dqr);
  ql_ip1 = q_i + dqm;
  qr_i = q_i - dqm;
}

static inline void PPM(Real q_im2, Real q_im1, Real q_i, Real q_ip1, Real q_ip2,
                       Real &ql_ip1, Real &qr_i) {
  const Real C2 = 1.25;
  Real qa = (q_i - q_im1);
  Real qb = (q_ip1 - q_i);
  const Real dd_im1 = 0.5 * qa + 0.5 * (q_im1 - q_im2);
  const Real dd = 0.5 * qb + 0.5 * qa;
  const Real dd_ip1 = 0.5 * (q_ip2 - q_ip1) + 0.5 * qb;
  Real dph = 0.5 * (q_im1 + q_i) + (dd_im1 - dd) / 6.0;
  Real dph_ip1 = 0.5 * (q_i + q_ip1) + (dd - dd_ip1) / 6.0;
  const Real d2qc_im1 = q_im2 + q_i - 2.0 * q_im1;
  const Real d2qc = q_im1 + q_ip1 - 2.0 * q_i;
  const Real d2qc_ip1 = q_i + q_ip2 - 2.0 * q_ip1;
  // i-1/2
  Real qa_tmp = dph - q_im1;
  Real qb_tmp = q_i - dph;
  qa = 3.0 * (q_im1 + q_i - 2.0 * dph);
  qb = d2qc_im1;
  Real qc = d2qc;
  Real qd = 0.0;
  if (SIGN(qa) == SIGN(qb) && SIGN(qa) == SIGN(qc)) {
    qd = SIGN(qa) * smin(C2 * std::abs(qb), smin(C2 * std::abs(qc), std::abs(qa)));
  }
  Real dph_tmp = 0.5 * (q_im1 + q_i) - qd / 6.0;
  if (qa_tmp * qb_tmp < 0.0) dph = dph_tmp;
  // i+1/2
  qa_tmp = dph_ip1 - q_i;
  qb_tmp = q_ip1 - dph_ip1;
  qa = 3.0 * (q_i + q_ip1 - 2.0 * dph_ip1);
  qb = d2qc;
  qc = d2qc_ip1;
  qd = 0.0;
  if (SIGN(qa) == SIGN(qb) && SIGN(qa) == SIGN(qc)) {
    qd = SIGN(qa) * smin(C2 * std::abs(qb), smin(C2 * std::abs(qc), std::abs(qa)));
  }
  Real dphip1_tmp = 0.5 * (q_i + q_ip1) - qd / 6.0;
  if (qa_tmp * qb_tmp < 0.0) dph_ip1 = dphip1_tmp;
  const Real d2qf = 6.0 * (dph + dph_ip1 - 2.0 * q_i);
  qr_i = dph;
  ql_ip1 = dph_ip1;
  const Real dqf_minus = q_i - qr_i;
  const Real dqf_plus = ql_ip1 - q_i;
  qa_tmp = dqf_minus * dqf_plus;
  qb_tmp = (q_ip1 - q_i) * (q_i - q_im1);
  qa = d2qc_im1;
  qb = d2qc;
  qc = d2qc_ip1;
  qd = d2qf;
  Real qe = 0.0;
  if (SIGN(qa) == SIGN(qb) && SIGN(qa) == SIGN(qc) && SIGN(qa) == SIGN(qd)) {
    qe = SIGN(qd) * smin(smin(C2 * std::abs(qa), C2 * std::abs(qb)),
                         smin(C2 * std::abs(qc), std::abs(qd)));
  }
  qa = smax(std::abs(q_im1), std::abs(q_im2));
  qb = smax(smax(std::abs(q_i), std::abs(q_ip1)), std::abs(q_ip2));
  Real rho = 0.0;
  if (std::abs(qd) > (1.0e-12) * smax(qa, qb)) rho = qe / qd;
  Real tmp_m = q_i - rho * dqf_minus;
  Real tmp_p = q_i + rho * dqf_plus;
  Real tmp2_m = q_i - 2.0 * dqf_plus;
  Real tmp2_p = q_i + 2.0 * dqf_minus;
  if ((qa_tmp <= 0.0 || qb_tmp <= 0.0)) {
    if (rho <= (1.0 - (1.0e-12))) {
      qr_i = tmp_m;
      ql_ip1 = tmp_p;
    }
  } else {
    if (std::abs(dqf_minus) >= 2.0 * std::abs(dqf_plus)) qr_i = tmp2_m;
    if (std::abs(dqf_plus) >= 2.0 * std::abs(dqf_minus)) ql_ip1 = tmp2_p;
  }
}

// Reconstruct nvar components of q along direction dir for the line through (k,j),
// cells lo..hi.  Following Reconstruct<recon,XNDIR>: for X1 the outputs land at
// ql[n][i+1], qr[n][i]; for X2/X3 at ql[n][i], qr[n][i] (i is the transverse index).
static void reconstruct(int recon, int dir, const Dims &d, const Real *q, int nvar, int k,
                        int j, int lo, int hi, std::vector<Real> &ql, std::vector<Real> &qr) {
  const ptrdiff_t s = (dir == 1) ? 1 : (dir == 2) ? d.ni : (ptrdiff_t)d.ni * d.nj;
  const size_t W = d.ni + 1;
  for (int n = 0; n < nvar; ++n) {
    for (int i = lo; i <= hi; ++i) {
      const Real *p = q + IX(d, n, k, j, i);
      Real *L = &ql[n * W + (dir == 1 ? i + 1 : i)];
      Real *R = &qr[n * W + i];
      if (recon == RECON_DC) {
        *L = *R = p[0];
      } else if (recon == RECON_PLM) {
        PLM(p[-s], p[0], p[s], *L, *R);
      } else {
        PPM(p[-2 * s], p[-s], p[0], p[s], p[2 * s], *L, *R);
      }
    }
  }
}

// ---- Riemann solvers: src/hydro/rsolvers/*.hpp --------------------------------
struct FluxOut {
  Real f[NHYDRO];
};

static inline void load_states(const std::vector<Real> &wl, const std::vector<Real> &wr,
                               size_t W, int i, int ivx, int ivy, int ivz, Real *wli,
                               Real *wri) {
  wli[IDN] = wl[IDN * W + i]; wli[IV1] = wl[ivx * W + i]; wli[IV2] = wl[ivy * W + i];
  wli[IV3] = wl[ivz * W + i]; wli[IPR] = wl[IPR * W + i];
  wri[IDN] = wr[IDN * W + i]; wri[IV1] = wr[ivx * W + i]; wri[IV2] = wr[ivy * W + i];
  wri[IV3] = wr[ivz * W + i]; wri[IPR] = wr[IPR * W + i];
}

// hydro_hlle.hpp:28-133
static void solve_hlle(const Real *wli, const Real *wri, Real gl0, Real gl1, Real gr0,
                       Real gr1, Real *flxi) {
  Real fl[NHYDRO], fr[NHYDRO];
  Real gammal = gl0, gammar = gr0;
  Real gm1l = gl1 - 1, gm1r = gr1 - 1;
  Real igm1l = 1.0 / gm1l, igm1r = 1.0 / gm1r;
  Real cl = C_LIGHT * std::sqrt(gammal / (1 + (igm1l + wli[IDN] * SQR(C_LIGHT) / wli[IPR])));
  Real cr = C_LIGHT * std::sqrt(gammar / (1 + (igm1r + wri[IDN] * SQR(C_LIGHT) / wri[IPR])));
  Real el = wli[IPR] * igm1l + 0.5 * wli[IDN] * (SQR(wli[IV1]) + SQR(wli[IV2]) + SQR(wli[IV3]));
  Real er = wri[IPR] * igm1r + 0.5 * wri[IDN] * (SQR(wri[IV1]) + SQR(wri[IV2]) + SQR(wri[IV3]));
  Real rhoa = .5 * (wli[IDN] + wri[IDN]);
  Real ca = .5 * (cl + cr);
  Real pmid = .5 * (wli[IPR] + wri[IPR] + (wli[IV1] - wri[IV1]) * rhoa * ca);
  Real ql = (pmid <= wli[IPR])
                ? 1.0
                : (1.0 + (gammal + 1) / std::sqrt(2 * gammal) * (pmid / wli[IPR] - 1.0));
  Real qr = (pmid <= wri[IPR])
                ? 1.0
                : (1.0 + (gammar + 1) / std::sqrt(2 * gammar) * (pmid / wri[IPR] - 1.0));
  Real al = wli[IV1] - cl * ql;
  Real ar = wri[IV1] + cr * qr;
  Real bp = ar > 0.0 ? ar : 0.0;
  Real bm = al < 0.0 ? al : 0.0;
  Real vxl = wli[IV1] - bm;
  Real vxr = wri[IV1] - bp;
  fl[IDN] = wli[IDN] * vxl;
  fr[IDN] = wri[IDN] * vxr;
  fl[IV1] = wli[IDN] * wli[IV1] * vxl;
  fr[IV1] = wri[IDN] * wri[IV1] * vxr;
  fl[IV2] = wli[IDN] * wli[IV2] * vxl;
  fr[IV2] = wri[IDN] * wri[IV2] * vxr;
  fl[IV3] = wli[IDN] * wli[IV3] * vxl;
  fr[IV3] = wri[IDN] * wri[IV3] * vxr;
  fl[IV1] += wli[IPR];
  fr[IV1] += wri[IPR];
  fl[IEN] = el * vxl + wli[IPR] * wli[IV1];
  fr[IEN] = er * vxr + wri[IPR] * wri[IV1];
  Real tmp = 0.0;
  if (bp != bm) tmp = 0.5 * (bp + bm) / (bp - bm);
  for (int n = 0; n < NHYDRO; ++n) flxi[n] = 0.5 * (fl[n] + fr[n]) + (fl[n] - fr[n]) * tmp;
}

// hydro_hllc.hpp:14-146 and hydro_lhllc.hpp:25-156 (low_mach selects the latter)
static void solve_hllc(const Real *wli, const Real *wri, Real gl0, Real gl1, Real gr0,
                       Real gr1, bool low_mach, Real *flxi) {
  Real fl[NHYDRO], fr[NHYDRO];
  Real gammal = gl0, gammar = gr0;
  Real gm1l = gl1 - 1, gm1r = gr1 - 1;
  Real igm1l = 1.0 / gm1l, igm1r = 1.0 / gm1r;
  Real cl = C_LIGHT * std::sqrt(gammal / (1 + (igm1l + wli[IDN] * SQR(C_LIGHT) / wli[IPR])));
  Real cr = C_LIGHT * std::sqrt(gammar / (1 + (igm1r + wri[IDN] * SQR(C_LIGHT) / wri[IPR])));
  Real el = wli[IPR] * igm1l + 0.5 * wli[IDN] * (SQR(wli[IV1]) + SQR(wli[IV2]) + SQR(wli[IV3]));
  Real er = wri[IPR] * igm1r + 0.5 * wri[IDN] * (SQR(wri[IV1]) + SQR(wri[IV2]) + SQR(wri[IV3]));
  Real rhoa = .5 * (wli[IDN] + wri[IDN]);
  Real ca = .5 * (cl + cr);
  Real pstar;
  if (!low_mach) {
    pstar = .5 * (wli[IPR] + wri[IPR]) - .5 * (wri[IV1] - wli[IV1]) * rhoa * ca;
  } else {
    Real machl = std::sqrt(wli[IV1] * wli[IV1] + wli[IV2] * wli[IV2] + wli[IV3] * wli[IV3]);
    Real machr = std::sqrt(wri[IV1] * wri[IV1] + wri[IV2] * wri[IV2] + wri[IV3] * wri[IV3]);
    Real chi = smax(machl, machr);
    Real phi = chi * (2.0 - chi);
    pstar = .5 * (wli[IPR] + wri[IPR]) - .5 * (wri[IV1] - wli[IV1]) * rhoa * ca * phi;
  }
  Real ql = (pstar <= wli[IPR])
                ? 1.0
                : std::sqrt(1.0 + (gammal + 1) / (2 * gammar) * (pstar / wli[IPR] - 1.0));
  Real qr = (pstar <= wri[IPR])
                ? 1.0
                : std::sqrt(1.0 + (gammal + 1) / (2 * gammar) * (pstar / wri[IPR] - 1.0));
  Real sl = wli[IV1] - cl * ql;
  Real sr = wri[IV1] + cr * qr;
  Real bp = sr > 0.0 ? sr : (TINY_NUMBER);
  Real bm = sl < 0.0 ? sl : -(TINY_NUMBER);
  Real vxl = wli[IV1] - sl;
  Real vxr = wri[IV1] - sr;
  Real tl = wli[IPR] + vxl * wli[IDN] * wli[IV1];
  Real tr = wri[IPR] + vxr * wri[IDN] * wri[IV1];
  Real ml = wli[IDN] * vxl;
  Real mr = -(wri[IDN] * vxr);
  Real sstar = (tl - tr) / (ml + mr);
  Real cp = (ml * tr + mr * tl) / (ml + mr);
  cp = cp > 0.0 ? cp : 0.0;
  vxl = wli[IV1] - bm;
  vxr = wri[IV1] - bp;
  fl[IDN] = wli[IDN] * vxl;
  fr[IDN] = wri[IDN] * vxr;
  fl[IV1] = wli[IDN] * wli[IV1] * vxl + wli[IPR];
  fr[IV1] = wri[IDN] * wri[IV1] * vxr + wri[IPR];
  fl[IV2] = wli[IDN] * wli[IV2] * vxl;
  fr[IV2] = wri[IDN] * wri[IV2] * vxr;
  fl[IV3] = wli[IDN] * wli[IV3] * vxl;
  fr[IV3] = wri[IDN] * wri[IV3] * vxr;
  fl[IEN] = el * vxl + wli[IPR] * wli[IV1];
  fr[IEN] = er * vxr + wri[IPR] * wri[IV1];
  Real ur, ul, ustar;
  if (sstar >= 0.0) {
    ul = sstar / (sstar - bm);
    ur = 0.0;
    ustar = -bm / (sstar - bm);
  } else {
    ul = 0.0;
    ur = -sstar / (bp - sstar);
    ustar = bp / (bp - sstar);
  }
  flxi[IDN] = ul * fl[IDN] + ur * fr[IDN];
  flxi[IV1] = ul * fl[IV1] + ur * fr[IV1] + ustar * cp;
  flxi[IV2] = ul * fl[IV2] + ur * fr[IV2];
  flxi[IV3] = ul * fl[IV3] + ur * fr[IV3];
  flxi[IEN] = ul * fl[IEN] + ur * fr[IEN] + ustar * cp * sstar;
}

// Riemann solve over the faces lo..hi of one line; writes cons.flux(ivx, ...).
static void riemann_line(int rsolver, int dir, const Dims &d, int k, int j, int lo, int hi,
                         const std::vector<Real> &wl, const std::vector<Real> &wr,
                         const std::vector<Real> &ifl, const std::vector<Real> &ifr,
                         Real *flux) {
  const int ivx = dir;  // IV1 + dir - 1
  const int ivy = IV1 + ((ivx - IV1) + 1) % 3;
  const int ivz = IV1 + ((ivx - IV1) + 2) % 3;
  const size_t W = d.ni + 1;
  const int nscalars = d.nvar - NHYDRO;
  for (int i = lo; i <= hi; ++i) {
    // face location in the flux array (k,j,i) with the marching index substituted
    Real wli[NHYDRO], wri[NHYDRO], flxi[NHYDRO];
    load_states(wl, wr, W, i, ivx, ivy, ivz, wli, wri);
    if (rsolver == RS_NONE) {
      for (int n = 0; n < NHYDRO; ++n) flxi[n] = 0.0;
    } else if (rsolver == RS_HLLE) {
      solve_hlle(wli, wri, ifl[0 * W + i], ifl[1 * W + i], ifr[0 * W + i], ifr[1 * W + i], flxi);
    } else {
      solve_hllc(wli, wri, ifl[0 * W + i], ifl[1 * W + i], ifr[0 * W + i], ifr[1 * W + i],
                 rsolver == RS_LHLLC, flxi);
    }
    flux[IX(d, IDN, k, j, i)] = flxi[IDN];
    flux[IX(d, ivx, k, j, i)] = flxi[IV1];
    flux[IX(d, ivy, k, j, i)] = flxi[IV2];
    flux[IX(d, ivz, k, j, i)] = flxi[IV3];
    flux[IX(d, IEN, k, j, i)] = flxi[IEN];
    // passive scalar fluxes: hydro.cpp:607-615
    for (int n = NHYDRO; n < NHYDRO + nscalars; ++n) {
      if (flux[IX(d, IDN, k, j, i)] >= 0.0)
        flux[IX(d, n, k, j, i)] = flux[IX(d, IDN, k, j, i)] * wl[n * W + i];
      else
        flux[IX(d, n, k, j, i)] = flux[IX(d, IDN, k, j, i)] * wr[n * W + i];
    }
  }
}

// CalculateFluxes<euler,recon,rsolver>: src/hydro/hydro.cpp:535-744, with the same
// row/column/plane ranges (fluxes on ghost rows included).
static void calculate_fluxes(const Dims &d, int recon, int rsolver, const Real *prim,
                             const Real *gamma, Real *flux1, Real *flux2, Real *flux3) {
  const int nvar = d.nvar;
  const size_t W = d.ni + 1;
  int jl = d.js, ju = d.je, kl = d.ks, ku = d.ke;
  if (d.ndim >= 2) {
    if (d.ndim == 2) { jl = d.js - 1; ju = d.je + 1; kl = d.ks; ku = d.ke; }
    else { jl = d.js - 1; ju = d.je + 1; kl = d.ks - 1; ku = d.ke + 1; }
  }
  // x1 flux
#pragma omp parallel
  {
    std::vector<Real> wl(nvar * W), wr(nvar * W), ifl(2 * W), ifr(2 * W);
#pragma omp for collapse(2) schedule(static)
    for (int k = kl; k <= ku; ++k)
      for (int j = jl; j <= ju; ++j) {
        reconstruct(recon, 1, d, prim, nvar, k, j, d.is - 1, d.ie + 1, wl, wr);
        reconstruct(recon, 1, d, gamma, 2, k, j, d.is - 1, d.ie + 1, ifl, ifr);
        riemann_line(rsolver, 1, d, k, j, d.is, d.ie + 1, wl, wr, ifl, ifr, flux1);
      }
  }
  if (d.ndim >= 2) {
    const int il = d.is - 1, iu = d.ie + 1;
    kl = (d.ndim == 2) ? d.ks : d.ks - 1;
    ku = (d.ndim == 2) ? d.ke : d.ke + 1;
#pragma omp parallel
    {
      std::vector<Real> wl(nvar * W), wr(nvar * W), wlb(nvar * W), ifl(2 * W), ifr(2 * W),
          iflb(2 * W);
#pragma omp for schedule(static)
      for (int k = kl; k <= ku; ++k) {
        for (int j = d.js - 1; j <= d.je + 1; ++j) {
          reconstruct(recon, 2, d, prim, nvar, k, j, il, iu, wlb, wr);
          reconstruct(recon, 2, d, gamma, 2, k, j, il, iu, iflb, ifr);
          if (j > d.js - 1) riemann_line(rsolver, 2, d, k, j, il, iu, wl, wr, ifl, ifr, flux2);
          std::swap(wl, wlb);
          std::swap(ifl, iflb);
        }
      }
    }
  }
  if (d.ndim >= 3) {
    const int il = d.is - 1, iu = d.ie + 1;
    jl = d.js - 1; ju = d.je + 1;
#pragma omp parallel
    {
      std::vector<Real> wl(nvar * W), wr(nvar * W), wlb(nvar * W), ifl(2 * W), ifr(2 * W),
          iflb(2 * W);
#pragma omp for schedule(static)
      for (int j = jl; j <= ju; ++j) {
        for (int k = d.ks - 1; k <= d.ke + 1; ++k) {
          reconstruct(recon, 3, d, prim, nvar, k, j, il, iu, wlb, wr);
          reconstruct(recon, 3, d, gamma, 2, k, j, il, iu, iflb, ifr);
          if (k > d.ks - 1) riemann_line(rsolver, 3, d, k, j, il, iu, wl, wr, ifl, ifr, flux3);
          std::swap(wl, wlb);
          std::swap(ifl, iflb);
        }
      }
    }
  }
}

// UpdateWithFluxDivergence (A3), interior cells, all nvar components.
static void update_with_flux_divergence(const Dims &d, Real *u0, const Real *u1,
                                        const Real *flux1, const Real *flux2,
                                        const Real *flux3, const Real *dx, Real gam0,
                                        Real gam1, Real beta_dt) {
  const Real a1 = dx[1] * dx[2], a2 = dx[0] * dx[2], a3 = dx[0] * dx[1];
  const Real vol = dx[0] * dx[1] * dx[2];
#pragma omp parallel for collapse(2) schedule(static)
  for (int n = 0; n < d.nvar; ++n)
    for (int k = d.ks; k <= d.ke; ++k)
      for (int j = d.js; j <= d.je; ++j)
        for (int i = d.is; i <= d.ie; ++i) {
          Real du = (a1 * flux1[IX(d, n, k, j, i + 1)] - a1 * flux1[IX(d, n, k, j, i)]);
          if (d.ndim >= 2)
            du += (a2 * flux2[IX(d, n, k, j + 1, i)] - a2 * flux2[IX(d, n, k, j, i)]);
          if (d.ndim == 3)
            du += (a3 * flux3[IX(d, n, k + 1, j, i)] - a3 * flux3[IX(d, n, k, j, i)]);
          const Real div = -du / vol;
          const size_t c = IX(d, n, k, j, i);
          u0[c] = gam0 * u0[c] + gam1 * u1[c] + beta_dt * div;
        }
}

// EstimateTimestep<euler>: src/hydro/hydro.cpp:351-420 (returns the min before cfl).
static Real estimate_timestep_min(const Dims &d, const Real *prim, const Real *cons,
                                  const Real *dx, Real gm1) {
  Real min_dt = std::numeric_limits<Real>::max();
#pragma omp parallel for collapse(2) reduction(min : min_dt) schedule(static)
  for (int k = d.ks; k <= d.ke; ++k)
    for (int j = d.js; j <= d.je; ++j)
      for (int i = d.is; i <= d.ie; ++i) {
        Real w[NHYDRO];
        for (int n = 0; n < NHYDRO; ++n) w[n] = prim[IX(d, n, k, j, i)];
        Real e_internal =
            (cons[IX(d, IEN, k, j, i)] - 0.5 * w[IDN] * (SQR(w[IV1]) + SQR(w[IV2]) + SQR(w[IV3]))) /
            w[IDN];
        Real bulkmod = eos_bulk_modulus(gm1, w[IDN], e_internal);
        const Real gamma_c = bulkmod / w[IPR];
        Real lam = C_LIGHT * std::sqrt(gamma_c / (1 + (e_internal + SQR(C_LIGHT)) * w[IDN] / w[IPR]));
        min_dt = std::fmin(min_dt, dx[0] / (std::fabs(w[IV1]) + lam));
        if (d.ndim > 1) min_dt = std::fmin(min_dt, dx[1] / (std::fabs(w[IV2]) + lam));
        if (d.ndim > 2) min_dt = std::fmin(min_dt, dx[2] / (std::fabs(w[IV3]) + lam));
      }
  return min_dt;
}

// ApplyGravity: src/gravity/gravity.cpp:374-410 for a constant field g (prim is the
// stale primitive state from the previous FillDerived, as in the reference).
static void apply_gravity(const Dims &d, Real *cons, const Real *prim, const Real *g, Real dt) {
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = d.ks; k <= d.ke; ++k)
    for (int j = d.js; j <= d.je; ++j)
      for (int i = d.is; i <= d.ie; ++i) {
        const Real rho = prim[IX(d, IDN, k, j, i)];
        cons[IX(d, IM1, k, j, i)] += g[0] * rho * dt;
        Real de = g[0] * prim[IX(d, IV1, k, j, i)];
        if (d.ndim >= 2) {
          cons[IX(d, IM2, k, j, i)] += g[1] * rho * dt;
          de += g[1] * prim[IX(d, IV2, k, j, i)];
        }
        if (d.ndim >= 3) {
          cons[IX(d, IM3, k, j, i)] += g[2] * rho * dt;
          de += g[2] * prim[IX(d, IV3, k, j, i)];
        }
        cons[IX(d, IEN, k, j, i)] += de * rho * dt;
      }
}

// ---- Uniform mesh of equal blocks + driver (A4-A6) ----------------------------
struct Mesh {
  Dims d;
  int nb[3];          // blocks per dimension
  int nblocks;
  int bc[3][2];       // per dim, inner/outer
  int recon, rsolver, integrator;
  Real gm1, cfl, dfloor, pfloor;
  Real dx[3];
  int gravity;
  Real g[3];
  std::vector<Real> u0, u1, prim, gamma, flux[3];
  Real time, dt, tlim;
  int ncycle;
};

static void stage_coeffs(int integrator, int stage, Real &gam0, Real &gam1, Real &beta) {
  if (integrator == INT_RK1) { gam0 = 0.0; gam1 = 1.0; beta = 1.0; }
  else if (integrator == INT_RK2) {
    if (stage == 1) { gam0 = 0.0; gam1 = 1.0; beta = 1.0; }
    else { gam0 = 0.5; gam1 = 0.5; beta = 0.5; }
  } else if (integrator == INT_RK3) {
    if (stage == 1) { gam0 = 0.0; gam1 = 1.0; beta = 1.0; }
    else if (stage == 2) { gam0 = 0.25; gam1 = 0.75; beta = 0.25; }
    else { gam0 = 2.0 / 3.0; gam1 = 1.0 / 3.0; beta = 2.0 / 3.0; }
  } else {  // vl2
    if (stage == 1) { gam0 = 0.0; gam1 = 1.0; beta = 0.5; }
    else { gam0 = 0.0; gam1 = 1.0; beta = 1.0; }
  }
}
static int nstages(int integrator) {
  return integrator == INT_RK1 ? 1 : integrator == INT_RK3 ? 3 : 2;
}

static inline int map_index(int g, int n, int bc_lo, int bc_hi, bool &flip) {
  if (g < 0) {
    if (bc_lo == BC_PERIODIC) return g + n;
    if (bc_lo == BC_OUTFLOW) return 0;
    flip = !flip;
    return -1 - g;
  }
  if (g >= n) {
    if (bc_hi == BC_PERIODIC) return g - n;
    if (bc_hi == BC_OUTFLOW) return n - 1;
    flip = !flip;
    return 2 * n - 1 - g;
  }
  return g;
}

// Fill every ghost cell of every block of field q (nvar components) from the
// global interior cell its per-dimension map points to (A6).
static void fill_ghosts(Mesh &m, std::vector<Real> &q) {
  const Dims &d = m.d;
  const int N[3] = {d.nx1 * m.nb[0], d.nx2 * m.nb[1], d.nx3 * m.nb[2]};
  const size_t bs = (size_t)d.nvar * d.ncell;
#pragma omp parallel for schedule(static)
  for (int b = 0; b < m.nblocks; ++b) {
    const int bi = b % m.nb[0], bj = (b / m.nb[0]) % m.nb[1], bk = b / (m.nb[0] * m.nb[1]);
    for (int k = 0; k < d.nk; ++k)
      for (int j = 0; j < d.nj; ++j)
        for (int i = 0; i < d.ni; ++i) {
          bool gi = (i < d.is || i > d.ie), gj = (j < d.js || j > d.je), gk = (k < d.ks || k > d.ke);
          if (!(gi || gj || gk)) continue;
          bool flip[3] = {false, false, false};
          int G[3];
          G[0] = map_index(bi * d.nx1 + (i - d.is), N[0], m.bc[0][0], m.bc[0][1], flip[0]);
          G[1] = (d.ndim >= 2) ? map_index(bj * d.nx2 + (j - d.js), N[1], m.bc[1][0], m.bc[1][1], flip[1]) : 0;
          G[2] = (d.ndim >= 3) ? map_index(bk * d.nx3 + (k - d.ks), N[2], m.bc[2][0], m.bc[2][1], flip[2]) : 0;
          const int sbi = G[0] / d.nx1, sbj = (d.ndim >= 2) ? G[1] / d.nx2 : 0,
                    sbk = (d.ndim >= 3) ? G[2] / d.nx3 : 0;
          const int sb = (sbk * m.nb[1] + sbj) * m.nb[0] + sbi;
          const int si = G[0] - sbi * d.nx1 + d.is;
          const int sj = (d.ndim >= 2) ? G[1] - sbj * d.nx2 + d.js : 0;
          const int sk = (d.ndim >= 3) ? G[2] - sbk * d.nx3 + d.ks : 0;
          for (int n = 0; n < d.nvar; ++n) {
            Real v = q[sb * bs + IX(d, n, sk, sj, si)];
            if ((n == IM1 && flip[0]) || (n == IM2 && flip[1]) || (n == IM3 && flip[2])) v = -v;
            q[b * bs + IX(d, n, k, j, i)] = v;
          }
        }
  }
}

static void fill_derived(Mesh &m) {
  const size_t bs = (size_t)m.d.nvar * m.d.ncell, gs = 2 * m.d.ncell;
  for (int b = 0; b < m.nblocks; ++b)
    cons_to_prim(m.d, &m.u0[b * bs], &m.prim[b * bs], &m.gamma[b * gs], m.gm1, m.dfloor, m.pfloor);
}

static Real estimate_dt(Mesh &m) {
  const size_t bs = (size_t)m.d.nvar * m.d.ncell;
  Real mn = std::numeric_limits<Real>::max();
  for (int b = 0; b < m.nblocks; ++b)
    mn = std::min(mn, m.cfl * estimate_timestep_min(m.d, &m.prim[b * bs], &m.u0[b * bs], m.dx, m.gm1));
  return mn;
}

// One RK step, stage order of ApophisDriver::MakeTaskCollection (apophis_driver.cpp:27-129).
static void step(Mesh &m, Real dt) {
  const Dims &d = m.d;
  const size_t bs = (size_t)d.nvar * d.ncell, gs = 2 * d.ncell;
  const int ns = nstages(m.integrator);
  for (int stage = 1; stage <= ns; ++stage) {
    if (stage == 1) m.u1 = m.u0;
    Real gam0, gam1, beta;
    stage_coeffs(m.integrator, stage, gam0, gam1, beta);
    const int recon = (m.integrator == INT_VL2 && stage == 1) ? RECON_DC : m.recon;
    for (int b = 0; b < m.nblocks; ++b) {
      calculate_fluxes(d, recon, m.rsolver, &m.prim[b * bs], &m.gamma[b * gs], &m.flux[0][b * bs],
                       d.ndim >= 2 ? &m.flux[1][b * bs] : nullptr,
                       d.ndim >= 3 ? &m.flux[2][b * bs] : nullptr);
      update_with_flux_divergence(d, &m.u0[b * bs], &m.u1[b * bs], &m.flux[0][b * bs],
                                  d.ndim >= 2 ? &m.flux[1][b * bs] : nullptr,
                                  d.ndim >= 3 ? &m.flux[2][b * bs] : nullptr, m.dx, gam0, gam1,
                                  beta * dt);
      if (m.gravity) apply_gravity(d, &m.u0[b * bs], &m.prim[b * bs], m.g, beta * dt);
    }
    fill_ghosts(m, m.u0);
    fill_derived(m);
  }
}


// ---- statically refined 2D mesh of uneven blocks -------------------------------------------
// The multi-level counterpart of the boundary exchange + flux correction that Parthenon does
// between levels (its prolongation/restriction and flux-correction code is not vendored,
// parity of these semantics against the reference is unpinned).  Restated here exactly as
// the CUDA path performs it:
//  * ghost cells across a face come from the neighbours' interiors only: same level: copy;
//    finer neighbour: average of the 2x2 fine cells, ((a+b)+(c+d))*0.25; coarser neighbour:
//    minmod-limited linear prolongation c + o_n*s_n + o_t*s_t (o = +-1/4 by the fine cell's
//    parity), s_n from the coarse neighbours along the normal (the one on the fine side is
//    the restricted average of the fine block's own edge cells), s_t from the coarse
//    block's transverse interior neighbours (0 at its edge); physical faces: outflow copy or
//    reflecting mirror with the normal momentum negated; corner ghosts copy the nearest
//    interior cell (no flux pass reads them);
//  * conservation at coarse-fine faces: after the x and y flux differences are summed, the
//    coarse boundary cell's difference is corrected from its own face flux F to the mean of
//    the two fine face fluxes Fn: du += a*F - a*Fn on a low face, a*Fn - a*F on a high face,
//    faces in the order x-, x+, y-, y+.
enum { FACE_SAME = 0, FACE_COARSER = 1, FACE_FINER = 2, FACE_BOUNDARY = 3 };

struct AmrBlock {
  int level, origin[2], nx[2];
  Real dx[3];
  int kind[4], cnt[4], nbr[4][4];
  Dims d;
  size_t off;  // first cell of the block in the flat pack
};

struct AmrMesh {
  int nvar = 5;  // 5 hydro variables, then the passive scalars
  int ng, recon, rsolver, integrator, bc[2][2], gravity;
  Real gm1, cfl, dfloor, pfloor, g[3];
  std::vector<AmrBlock> blocks;
  size_t total = 0;
  std::vector<Real> u0, u1, prim, gamma, flux[2], du;
  std::vector<size_t> du_off;
  Real time = 0, dt = 0;
  int ncycle = 0;
  int plant_no_correction = 0;  // tests only: skip the coarse-fine flux correction
};

static inline size_t ACELL(const AmrBlock &B, int d, int a, int t) {
  // entire-domain cell of interior normal index a (along d) and transverse index t
  const int i = d == 0 ? B.d.ng + a : B.d.ng + t;
  const int j = d == 0 ? B.d.ng + t : B.d.ng + a;
  return (size_t)j * B.d.ni + i;
}
static inline Real AU(const AmrMesh &m, const std::vector<Real> &q, const AmrBlock &B, int v,
                      size_t cell) {
  return q[B.off * m.nvar + (size_t)v * B.d.ncell + cell];
}
static inline Real minmod(Real a, Real b) {
  if (!(a * b > 0.0)) return 0.0;
  return (std::abs(a) < std::abs(b)) ? a : b;
}

// Ghost value of all nvar components for face (d, s) of block B at depth k, transverse index t.
static void amr_ghost(const AmrMesh &m, const std::vector<Real> &q, const AmrBlock &B, int d,
                      int s, int k, int t, Real *out) {
  const int face = 2 * d + s, td = 1 - d;
  const int kind = B.kind[face];
  if (kind == FACE_SAME) {
    const AmrBlock &N = m.blocks[B.nbr[face][0]];
    const int a = s == 0 ? N.nx[d] - 1 - k : k;
    const int tn = B.origin[td] + t - N.origin[td];
    for (int v = 0; v < m.nvar; ++v) out[v] = AU(m, q, N, v, ACELL(N, d, a, tn));
  } else if (kind == FACE_BOUNDARY) {
    const int bcv = m.bc[d][s];
    if (bcv == BC_OUTFLOW) {
      const int a = s == 0 ? 0 : B.nx[d] - 1;
      for (int v = 0; v < m.nvar; ++v) out[v] = AU(m, q, B, v, ACELL(B, d, a, t));
    } else {
      const int a = s == 0 ? k : B.nx[d] - 1 - k;
      for (int v = 0; v < m.nvar; ++v) {
        const Real x = AU(m, q, B, v, ACELL(B, d, a, t));
        out[v] = (v == 1 + d) ? -x : x;
      }
    }
  } else if (kind == FACE_FINER) {
    const int tg2 = 2 * (B.origin[td] + t);
    const AmrBlock *F = nullptr;
    for (int n = 0; n < B.cnt[face]; ++n) {
      const AmrBlock &C = m.blocks[B.nbr[face][n]];
      if (tg2 >= C.origin[td] && tg2 < C.origin[td] + C.nx[td]) F = &C;
    }
    const int ft = tg2 - F->origin[td];
    const int a0 = s == 0 ? F->nx[d] - 1 - 2 * k : 2 * k;
    const int a1 = s == 0 ? a0 - 1 : a0 + 1;
    for (int v = 0; v < m.nvar; ++v)
      out[v] = ((AU(m, q, *F, v, ACELL(*F, d, a0, ft)) + AU(m, q, *F, v, ACELL(*F, d, a0, ft + 1))) +
                (AU(m, q, *F, v, ACELL(*F, d, a1, ft)) + AU(m, q, *F, v, ACELL(*F, d, a1, ft + 1)))) *
               0.25;
  } else {  // COARSER
    const AmrBlock &C = m.blocks[B.nbr[face][0]];
    const int tg = B.origin[td] + t;
    const int tc = (tg >> 1) - C.origin[td];
    const int kc = k >> 1;
    const int ic = s == 0 ? C.nx[d] - 1 - kc : kc;  // coarse normal index
    // fine global normal index of the ghost and its coarse parent
    const int gf = s == 0 ? B.origin[d] - 1 - k : B.origin[d] + B.nx[d] + k;
    const Real on = (gf & 1) ? 0.25 : -0.25;
    const Real ot = (tg & 1) ? 0.25 : -0.25;
    for (int v = 0; v < m.nvar; ++v) {
      const Real c = AU(m, q, C, v, ACELL(C, d, ic, tc));
      // neighbours along +d / -d in the coarse block's index space
      Real cm, cp;
      const int tf0 = 2 * (tc + C.origin[td]) - B.origin[td];  // fine transverse pair in B
      auto restricted = [&](int a0, int a1) {
        return ((AU(m, q, B, v, ACELL(B, d, a0, tf0)) + AU(m, q, B, v, ACELL(B, d, a0, tf0 + 1))) +
                (AU(m, q, B, v, ACELL(B, d, a1, tf0)) + AU(m, q, B, v, ACELL(B, d, a1, tf0 + 1)))) *
               0.25;
      };
      if (s == 0) {  // B lies on the +d side of C
        cm = AU(m, q, C, v, ACELL(C, d, ic - 1, tc));
        cp = ic + 1 < C.nx[d] ? AU(m, q, C, v, ACELL(C, d, ic + 1, tc)) : restricted(0, 1);
      } else {       // B lies on the -d side of C
        cm = ic - 1 >= 0 ? AU(m, q, C, v, ACELL(C, d, ic - 1, tc))
                         : restricted(B.nx[d] - 1, B.nx[d] - 2);
        cp = AU(m, q, C, v, ACELL(C, d, ic + 1, tc));
      }
      const Real sn = minmod(c - cm, cp - c);
      Real st = 0.0;
      if (tc - 1 >= 0 && tc + 1 < C.nx[td])
        st = minmod(c - AU(m, q, C, v, ACELL(C, d, ic, tc - 1)), AU(m, q, C, v, ACELL(C, d, ic, tc + 1)) - c);
      out[v] = c + on * sn + ot * st;
    }
  }
}

static void amr_fill_ghosts(AmrMesh &m, std::vector<Real> &q) {
  // reads interiors only, writes ghosts only
#pragma omp parallel for schedule(dynamic, 4)
  for (int b = 0; b < (int)m.blocks.size(); ++b) {
    const AmrBlock &B = m.blocks[b];
    const Dims &d = B.d;
    Real val[64];
    for (int j = 0; j < d.nj; ++j)
      for (int i = 0; i < d.ni; ++i) {
        const bool gi = i < d.ng || i >= d.ng + B.nx[0];
        const bool gj = j < d.ng || j >= d.ng + B.nx[1];
        if (!gi && !gj) continue;
        const size_t cell = (size_t)j * d.ni + i;
        if (gi && gj) {
          const int ci = std::min(std::max(i, d.ng), d.ng + B.nx[0] - 1);
          const int cj = std::min(std::max(j, d.ng), d.ng + B.nx[1] - 1);
          for (int v = 0; v < m.nvar; ++v) val[v] = AU(m, q, B, v, (size_t)cj * d.ni + ci);
        } else if (gi) {
          const int s = i < d.ng ? 0 : 1;
          const int k = s == 0 ? d.ng - 1 - i : i - (d.ng + B.nx[0]);
          amr_ghost(m, q, B, 0, s, k, j - d.ng, val);
        } else {
          const int s = j < d.ng ? 0 : 1;
          const int k = s == 0 ? d.ng - 1 - j : j - (d.ng + B.nx[1]);
          amr_ghost(m, q, B, 1, s, k, i - d.ng, val);
        }
        for (int v = 0; v < m.nvar; ++v) q[B.off * m.nvar + (size_t)v * d.ncell + cell] = val[v];
      }
  }
}

static void amr_fill_derived(AmrMesh &m) {
  for (const AmrBlock &B : m.blocks)
    cons_to_prim(B.d, &m.u0[B.off * m.nvar], &m.prim[B.off * m.nvar], &m.gamma[B.off * 2], m.gm1, m.dfloor, m.pfloor);
}

static Real amr_estimate_dt(AmrMesh &m) {
  Real mn = std::numeric_limits<Real>::max();
  for (AmrBlock &B : m.blocks)
    mn = std::min(mn, m.cfl * estimate_timestep_min(B.d, &m.prim[B.off * m.nvar], &m.u0[B.off * m.nvar], B.dx, m.gm1));
  return mn;
}

static void amr_step(AmrMesh &m, Real dt) {
  const int ns = nstages(m.integrator);
  for (int stage = 1; stage <= ns; ++stage) {
    if (stage == 1) m.u1 = m.u0;
    Real gam0, gam1, beta;
    stage_coeffs(m.integrator, stage, gam0, gam1, beta);
    const int recon = (m.integrator == INT_VL2 && stage == 1) ? RECON_DC : m.recon;
    const int nb = (int)m.blocks.size();
    for (int b = 0; b < nb; ++b) {
      AmrBlock &B = m.blocks[b];
      calculate_fluxes(B.d, recon, m.rsolver, &m.prim[B.off * m.nvar], &m.gamma[B.off * 2],
                       &m.flux[0][B.off * m.nvar], &m.flux[1][B.off * m.nvar], nullptr);
    }
    // flux differences, x then y
#pragma omp parallel for schedule(dynamic, 4)
    for (int b = 0; b < nb; ++b) {
      AmrBlock &B = m.blocks[b];
      const Dims &d = B.d;
      const Real a1 = B.dx[1] * B.dx[2], a2 = B.dx[0] * B.dx[2];
      const Real *F1 = &m.flux[0][B.off * m.nvar], *F2 = &m.flux[1][B.off * m.nvar];
      Real *du = &m.du[m.du_off[b]];
      const size_t nint = (size_t)B.nx[0] * B.nx[1];
      for (int v = 0; v < m.nvar; ++v)
        for (int j = 0; j < B.nx[1]; ++j)
          for (int i = 0; i < B.nx[0]; ++i) {
            const size_t c = IX(d, v, 0, j + d.ng, i + d.ng);
            Real x = (a1 * F1[c + 1] - a1 * F1[c]);
            x += (a2 * F2[c + d.ni] - a2 * F2[c]);
            du[v * nint + (size_t)j * B.nx[0] + i] = x;
          }
    }
    // conservation at coarse-fine faces
#pragma omp parallel for schedule(dynamic, 4)
    for (int b = 0; b < nb; ++b) {
      AmrBlock &B = m.blocks[b];
      Real *du = &m.du[m.du_off[b]];
      const size_t nint = (size_t)B.nx[0] * B.nx[1];
      for (int face = 0; face < 4; ++face) {
        if (B.kind[face] != FACE_FINER || m.plant_no_correction) continue;
        const int d = face / 2, s = face % 2, td = 1 - d;
        const Real area = d == 0 ? B.dx[1] * B.dx[2] : B.dx[0] * B.dx[2];
        const Real *Fb = &m.flux[d][B.off * m.nvar];
        for (int t = 0; t < B.nx[td]; ++t) {
          const int tg2 = 2 * (B.origin[td] + t);
          const AmrBlock *F = nullptr;
          for (int n = 0; n < B.cnt[face]; ++n) {
            const AmrBlock &C = m.blocks[B.nbr[face][n]];
            if (tg2 >= C.origin[td] && tg2 < C.origin[td] + C.nx[td]) F = &C;
          }
          const int ft = tg2 - F->origin[td];
          const Real *Ff = &m.flux[d][F->off * m.nvar];
          // face index (along d) of the shared face in each block
          const int fb = s == 0 ? 0 : B.nx[d];
          const int ff = s == 0 ? F->nx[d] : 0;
          const int a = s == 0 ? 0 : B.nx[d] - 1;  // coarse boundary cell
          for (int v = 0; v < m.nvar; ++v) {
            auto fidx = [&](const AmrBlock &X, int fa, int tt) {
              const int i = d == 0 ? X.d.ng + fa : X.d.ng + tt;
              const int j = d == 0 ? X.d.ng + tt : X.d.ng + fa;
              return (size_t)v * X.d.ncell + (size_t)j * X.d.ni + i;
            };
            const Real Fold = Fb[fidx(B, fb, t)];
            const Real Fnew = 0.5 * (Ff[fidx(*F, ff, ft)] + Ff[fidx(*F, ff, ft + 1)]);
            const int i = d == 0 ? a : t, j = d == 0 ? t : a;
            Real &x = du[v * nint + (size_t)j * B.nx[0] + i];
            x = s == 0 ? x + (area * Fold - area * Fnew) : x + (area * Fnew - area * Fold);
          }
        }
      }
    }
    // update, gravity
#pragma omp parallel for schedule(dynamic, 4)
    for (int b = 0; b < nb; ++b) {
      AmrBlock &B = m.blocks[b];
      const Dims &d = B.d;
      const Real vol = B.dx[0] * B.dx[1] * B.dx[2];
      const Real *du = &m.du[m.du_off[b]];
      const size_t nint = (size_t)B.nx[0] * B.nx[1];
      Real *u0 = &m.u0[B.off * m.nvar];
      const Real *u1 = &m.u1[B.off * m.nvar];
      for (int v = 0; v < m.nvar; ++v)
        for (int j = 0; j < B.nx[1]; ++j)
          for (int i = 0; i < B.nx[0]; ++i) {
            const size_t c = IX(d, v, 0, j + d.ng, i + d.ng);
            const Real div = -du[v * nint + (size_t)j * B.nx[0] + i] / vol;
            u0[c] = gam0 * u0[c] + gam1 * u1[c] + beta * dt * div;
          }
      if (m.gravity) apply_gravity(d, u0, &m.prim[B.off * m.nvar], m.g, beta * dt);
    }
    amr_fill_ghosts(m, m.u0);
    amr_fill_derived(m);
  }
}

}  // namespace orc

using namespace orc;

extern "C" {

// ---- single-block kernels (arrays are (nvar, nk, nj, ni), ghosts included) ----
void orc_cons_to_prim(double *cons, double *prim, double *gamma, int nvar, int nx1, int nx2,
                      int nx3, int ng, int ndim, double gm1, double dfloor, double pfloor) {
  Dims d = make_dims(nvar, nx1, nx2, nx3, ng, ndim);
  cons_to_prim(d, cons, prim, gamma, gm1, dfloor, pfloor);
}

void orc_calculate_fluxes(const double *prim, const double *gamma, double *flux1, double *flux2,
                          double *flux3, int nvar, int nx1, int nx2, int nx3, int ng, int ndim,
                          int recon, int rsolver) {
  Dims d = make_dims(nvar, nx1, nx2, nx3, ng, ndim);
  calculate_fluxes(d, recon, rsolver, prim, gamma, flux1, flux2, flux3);
}

void orc_update(double *u0, const double *u1, const double *flux1, const double *flux2,
                const double *flux3, int nvar, int nx1, int nx2, int nx3, int ng, int ndim,
                const double *dx, double gam0, double gam1, double beta_dt) {
  Dims d = make_dims(nvar, nx1, nx2, nx3, ng, ndim);
  update_with_flux_divergence(d, u0, u1, flux1, flux2, flux3, dx, gam0, gam1, beta_dt);
}

double orc_estimate_dt(const double *prim, const double *cons, int nvar, int nx1, int nx2,
                       int nx3, int ng, int ndim, const double *dx, double cfl, double gm1) {
  Dims d = make_dims(nvar, nx1, nx2, nx3, ng, ndim);
  return cfl * estimate_timestep_min(d, prim, cons, dx, gm1);
}

void orc_apply_gravity(double *cons, const double *prim, int nvar, int nx1, int nx2, int nx3,
                       int ng, int ndim, const double *g, double dt) {
  Dims d = make_dims(nvar, nx1, nx2, nx3, ng, ndim);
  apply_gravity(d, cons, prim, g, dt);
}

// Single-function restatements, exposed for known-answer tests.
void orc_plm(double a, double b, double c, double *ql_ip1, double *qr_i) { PLM(a, b, c, *ql_ip1, *qr_i); }
void orc_ppm(double a, double b, double c, double e, double f, double *ql_ip1, double *qr_i) {
  PPM(a, b, c, e, f, *ql_ip1, *qr_i);
}
// n stencils at once: q (n, 3) or (n, 5) -> out (n, 2) = (ql_{i+1}, qr_i)
void orc_plm_many(const double *q, double *out, long n) {
  for (long s = 0; s < n; ++s) PLM(q[3 * s], q[3 * s + 1], q[3 * s + 2], out[2 * s], out[2 * s + 1]);
}
void orc_ppm_many(const double *q, double *out, long n) {
  for (long s = 0; s < n; ++s)
    PPM(q[5 * s], q[5 * s + 1], q[5 * s + 2], q[5 * s + 3], q[5 * s + 4], out[2 * s], out[2 * s + 1]);
}
// wl, wr: (rho, vx, vy, vz, p) with vx the face-normal velocity; g*: (gamma_c, gamma_e)
void orc_riemann(int rsolver, const double *wl, const double *wr, const double *gl,
                 const double *gr, double *flx) {
  if (rsolver == RS_HLLE) solve_hlle(wl, wr, gl[0], gl[1], gr[0], gr[1], flx);
  else if (rsolver == RS_NONE) for (int n = 0; n < NHYDRO; ++n) flx[n] = 0.0;
  else solve_hllc(wl, wr, gl[0], gl[1], gr[0], gr[1], rsolver == RS_LHLLC, flx);
}

// ---- uniform mesh driver ----------------------------------------------------------
// ints: [nvar, ndim, nx1, nx2, nx3 (block), nb1, nb2, nb3, ng, recon, rsolver, integrator,
//        bc x1i, x1o, x2i, x2o, x3i, x3o, gravity]
// reals: [gm1, cfl, dfloor, pfloor, dx1, dx2, dx3, g1, g2, g3]
void *orc_mesh_create(const int *ints, const double *reals) {
  Mesh *m = new Mesh();
  m->d = make_dims(ints[0], ints[2], ints[3], ints[4], ints[8], ints[1]);
  m->nb[0] = ints[5]; m->nb[1] = ints[6]; m->nb[2] = ints[7];
  m->nblocks = m->nb[0] * m->nb[1] * m->nb[2];
  m->recon = ints[9]; m->rsolver = ints[10]; m->integrator = ints[11];
  for (int dd = 0; dd < 3; ++dd) { m->bc[dd][0] = ints[12 + 2 * dd]; m->bc[dd][1] = ints[13 + 2 * dd]; }
  m->gravity = ints[18];
  m->gm1 = reals[0]; m->cfl = reals[1]; m->dfloor = reals[2]; m->pfloor = reals[3];
  for (int dd = 0; dd < 3; ++dd) { m->dx[dd] = reals[4 + dd]; m->g[dd] = reals[7 + dd]; }
  const size_t n = (size_t)m->nblocks * m->d.nvar * m->d.ncell;
  m->u0.assign(n, 0.0); m->u1.assign(n, 0.0); m->prim.assign(n, 0.0);
  m->gamma.assign((size_t)m->nblocks * 2 * m->d.ncell, 0.0);
  for (int dd = 0; dd < 3; ++dd) m->flux[dd].assign(n, 0.0);
  m->time = 0.0; m->dt = 0.0; m->tlim = 1e300; m->ncycle = 0;
  return m;
}

void orc_mesh_destroy(void *h) { delete (Mesh *)h; }

// Load conserved variables (interior values used; ghosts refilled), then
// FillDerived and the initial dt estimate.
void orc_mesh_set_cons(void *h, const double *cons) {
  Mesh &m = *(Mesh *)h;
  std::memcpy(m.u0.data(), cons, m.u0.size() * sizeof(double));
  fill_ghosts(m, m.u0);
  fill_derived(m);
  m.dt = estimate_dt(m);
}

void orc_mesh_get(void *h, int what, double *out) {
  Mesh &m = *(Mesh *)h;
  const std::vector<Real> *v = what == 0 ? &m.u0 : what == 1 ? &m.prim : what == 2 ? &m.gamma
                              : what == 3 ? &m.u1 : &m.flux[what - 4];
  std::memcpy(out, v->data(), v->size() * sizeof(double));
}

// Advance up to nsteps cycles (or until tlim), with the dt policy (A5) unless
// fixed_dt > 0, in which case every step uses fixed_dt.  Returns cycles taken.
int orc_mesh_run(void *h, int nsteps, double tlim, double fixed_dt) {
  Mesh &m = *(Mesh *)h;
  int taken = 0;
  while (taken < nsteps && m.time < tlim) {
    Real dt = fixed_dt > 0 ? fixed_dt : m.dt;
    if (fixed_dt <= 0 && m.time < tlim && (tlim - m.time) < dt) dt = tlim - m.time;
    step(m, dt);
    m.time += dt;
    m.ncycle++;
    taken++;
    const Real est = estimate_dt(m);
    m.dt = std::min(2.0 * dt, est);
  }
  return taken;
}

void orc_mesh_state(void *h, double *out3) {
  Mesh &m = *(Mesh *)h;
  out3[0] = m.time; out3[1] = m.dt; out3[2] = m.ncycle;
}


// ---- refined mesh driver ------------------------------------------------------------------
// ints: [nblocks, ng, recon, rsolver, integrator, bc x1i, x1o, x2i, x2o, gravity, nvar]
// blk (per block 1+2+2+4+4+16 = 29 ints): level, origin[2], nx[2], kind[4], cnt[4], nbr[4][4]
// reals: [gm1, cfl, dfloor, pfloor, g1, g2, g3]; bdx: per block dx1, dx2, dx3
void *orc_amr_create(const int *ints, const int *blk, const double *reals, const double *bdx) {
  AmrMesh *m = new AmrMesh();
  const int nb = ints[0];
  m->ng = ints[1]; m->recon = ints[2]; m->rsolver = ints[3]; m->integrator = ints[4];
  m->bc[0][0] = ints[5]; m->bc[0][1] = ints[6]; m->bc[1][0] = ints[7]; m->bc[1][1] = ints[8];
  m->gravity = ints[9];
  m->nvar = ints[10];
  const int nv = m->nvar;
  m->gm1 = reals[0]; m->cfl = reals[1]; m->dfloor = reals[2]; m->pfloor = reals[3];
  for (int d = 0; d < 3; ++d) m->g[d] = reals[4 + d];
  m->blocks.resize(nb);
  size_t off = 0, doff = 0;
  for (int b = 0; b < nb; ++b) {
    AmrBlock &B = m->blocks[b];
    const int *p = blk + 29 * b;  // level, origin[2], nx[2], kind[4], cnt[4], nbr[4][4]
    B.level = p[0]; B.origin[0] = p[1]; B.origin[1] = p[2]; B.nx[0] = p[3]; B.nx[1] = p[4];
    for (int f = 0; f < 4; ++f) { B.kind[f] = p[5 + f]; B.cnt[f] = p[9 + f]; }
    for (int f = 0; f < 4; ++f) for (int n = 0; n < 4; ++n) B.nbr[f][n] = p[13 + 4 * f + n];
    for (int d = 0; d < 3; ++d) B.dx[d] = bdx[3 * b + d];
    B.d = make_dims(nv, B.nx[0], B.nx[1], 1, m->ng, 2);
    B.off = off;
    off += B.d.ncell;
    m->du_off.push_back(doff);
    doff += (size_t)nv * B.nx[0] * B.nx[1];
  }
  m->total = off;
  m->u0.assign(nv * off, 0.0); m->u1.assign(nv * off, 0.0); m->prim.assign(nv * off, 0.0);
  m->gamma.assign(2 * off, 0.0); m->flux[0].assign(nv * off, 0.0); m->flux[1].assign(nv * off, 0.0);
  m->du.assign(doff, 0.0);
  return m;
}

void orc_amr_destroy(void *h) { delete (AmrMesh *)h; }

// Plants a mistake for the tests: the step skips the coarse-fine flux correction.
void orc_amr_plant_no_correction(void *h) { ((AmrMesh *)h)->plant_no_correction = 1; }

void orc_amr_set_cons(void *h, const double *cons) {
  AmrMesh &m = *(AmrMesh *)h;
  std::memcpy(m.u0.data(), cons, m.u0.size() * sizeof(double));
  amr_fill_ghosts(m, m.u0);
  amr_fill_derived(m);
  m.dt = amr_estimate_dt(m);
}

void orc_amr_get(void *h, int what, double *out) {
  AmrMesh &m = *(AmrMesh *)h;
  const std::vector<Real> &v = what == 0 ? m.u0 : m.prim;
  std::memcpy(out, v.data(), v.size() * sizeof(double));
}

int orc_amr_run(void *h, int nsteps, double tlim, double fixed_dt) {
  AmrMesh &m = *(AmrMesh *)h;
  int taken = 0;
  while (taken < nsteps && m.time < tlim) {
    Real dt = fixed_dt > 0 ? fixed_dt : m.dt;
    if (fixed_dt <= 0 && (tlim - m.time) < dt) dt = tlim - m.time;
    amr_step(m, dt);
    m.time += dt;
    m.ncycle++;
    taken++;
    m.dt = std::min(2.0 * dt, amr_estimate_dt(m));
  }
  return taken;
}

void orc_amr_state(void *h, double *out3) {
  AmrMesh &m = *(AmrMesh *)h;
  out3[0] = m.time; out3[1] = m.dt; out3[2] = m.ncycle;
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void orc_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

}  // extern "C"
