// aph_math.cuh -- device arithmetic of the hydro flux path (sm_103a).
//
// On GB300 every FP64 instruction -- add, mul, fma, but also compare (DSETP) and
// min/max -- goes through a pipe that retires about two warp-lanes per clock per SM,
// while the integer and FP32 pipes run about sixty times faster.  The predicates and
// min/max below therefore work on the IEEE bit patterns with integer instructions.
// They give the same answer as the IEEE comparison for every non-NaN input, -0.0 and
// +0.0 included, so using them changes no result bit.
//
// APH_EXACT selects the arithmetic:
//   1  the reference's operation order, one rounding per operation (the translation
//      unit is built with --fmad=false); bit-identical to the reference's FP64 CPU path.
//   0  the same algorithm with fused multiply-adds, shared reciprocals and
//      precomputed gamma-dependent constants; agrees to ~1e-15 relative per operation.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#ifndef APH_EXACT
#define APH_EXACT 0
#endif

namespace aph {

constexpr int IDN = 0, IM1 = 1, IM2 = 2, IM3 = 3, IEN = 4, NHYDRO = 5;
constexpr int IV1 = 1, IV2 = 2, IV3 = 3, IPR = 4;
constexpr int RECON_DC = 1, RECON_PLM = 2, RECON_PPM = 3;
constexpr int RS_NONE = 1, RS_HLLE = 2, RS_HLLC = 3, RS_LHLLC = 4;

constexpr double C_LIGHT = 2.99792458e10;        // hydro_hlle.hpp:26
constexpr double C_LIGHT2 = C_LIGHT * C_LIGHT;   // SQR(C_LIGHT)
constexpr double TINY_NUMBER = 1.0e-20;
constexpr double PPM_C2 = 1.25;                  // ppm_simple.hpp:36

// ---- integer-pipe predicates ------------------------------------------------
__device__ __forceinline__ bool is_neg(double x) {  // x < 0.0
  const int hi = __double2hiint(x), lo = __double2loint(x);
  return hi < 0 && ((((unsigned)hi) << 1) | (unsigned)lo) != 0u;
}
__device__ __forceinline__ bool is_pos(double x) {  // x > 0.0
  const int hi = __double2hiint(x), lo = __double2loint(x);
  return hi >= 0 && (hi | lo) != 0;
}
// monotone integer key: a < b  <=>  okey(a) < okey(b)  (-0.0 and +0.0 share key 0)
__device__ __forceinline__ long long okey(double x) {
  const long long b = __double_as_longlong(x);
  return b >= 0 ? b : (long long)(0x8000000000000000ULL - (unsigned long long)b);
}
__device__ __forceinline__ bool lt(double a, double b) { return okey(a) < okey(b); }
__device__ __forceinline__ bool le(double a, double b) { return okey(a) <= okey(b); }
__device__ __forceinline__ bool gt(double a, double b) { return okey(a) > okey(b); }
// std::min / std::max tie rules (the first argument wins when neither is smaller)
__device__ __forceinline__ double smin(double a, double b) { return lt(b, a) ? b : a; }
__device__ __forceinline__ double smax(double a, double b) { return lt(a, b) ? b : a; }
__device__ __forceinline__ unsigned long long mag(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffULL;
}
__device__ __forceinline__ double dabs(double x) { return __longlong_as_double((long long)mag(x)); }
// bits of 2*|x| (exact doubling: exponent +1, or a shift for subnormals; overflow -> inf)
__device__ __forceinline__ unsigned long long twice_mag(double x) {
  const unsigned long long m = mag(x);
  const unsigned long long e = m >> 52;
  if (e == 0) return m << 1;
  if (e >= 0x7feULL) return 0x7ff0000000000000ULL;
  return m + (1ULL << 52);
}
// v with its sign flipped when neg (SIGN(s) * v for SIGN in {-1, +1})
__device__ __forceinline__ double flip_if(double v, bool neg) {
  return neg ? __longlong_as_double(__double_as_longlong(v) ^ (long long)0x8000000000000000ULL) : v;
}
__device__ __forceinline__ double from_bits(unsigned long long b) { return __longlong_as_double((long long)b); }
// b strictly between a and c: the reference's sign test (b - a) * (c - b) > 0 without the FP64
// subtractions and product (a difference of finite doubles is zero only when they are
// equal; the two differ only where the product underflows to zero, for differences of
// order 1e-162).  Fast mode.
__device__ __forceinline__ bool strictly_between(double a, double b, double c) {
  const long long ka = okey(a), kb = okey(b), kc = okey(c);
  return (ka < kb && kb < kc) || (ka > kb && kb > kc);
}
// x beyond both a and b on the same side: the sign test (x - a) * (b - x) < 0.  Fast mode.
__device__ __forceinline__ bool strictly_outside(double x, double a, double b) {
  const long long kx = okey(x), ka = okey(a), kb = okey(b);
  return (kx > ka && kx > kb) || (kx < ka && kx < kb);
}

// ---- exact operations on the integer pipe for tame operands -------------------------
// A value is tame when it is zero or a normal number with 2^-200 <= |x| < 2^201.  The
// reconstruction of a window of tame values only forms sums, differences and a few
// products and quotients of them, which stay zero or normal far from the underflow and
// overflow thresholds (a nonzero difference of tame values is at least 2^-252).  For those
// values the operations below give exactly the bits of the FP64 operation they replace:
//   half_x(x) == 0.5 * x and twice_x(x) == 2.0 * x (an exponent step; zero kept),
//   div6_x(x) == x / 6.0 (correctly rounded, see below),
// and the sign of a product of two differences is the product of their signs (no product
// underflows), which strictly_between / strictly_outside decide on the integer pipe.
__device__ __forceinline__ bool tame(double x) {
  const unsigned hi = (unsigned)__double2hiint(x) & 0x7fffffffu;
  const unsigned e = hi >> 20;  // biased exponent
  return (e - (1023u - 200u) <= 400u) || ((hi | (unsigned)__double2loint(x)) == 0u);
}
__device__ __forceinline__ bool tame_nz(double x) {  // tame and nonzero
  const unsigned e = ((unsigned)__double2hiint(x) & 0x7fffffffu) >> 20;
  return e - (1023u - 200u) <= 400u;
}
__device__ __forceinline__ double half_x(double x) {
  const long long b = __double_as_longlong(x);
  return (b << 1) == 0 ? x : __longlong_as_double(b - (1LL << 52));
}
__device__ __forceinline__ double twice_x(double x) {
  const long long b = __double_as_longlong(x);
  return (b << 1) == 0 ? x : __longlong_as_double(b + (1LL << 52));
}
// x / 6.0 correctly rounded, on the integer pipe: with the significand M (leading 1 moved to
// bit 63), floor(M / 3) is the high word of M * 0xAAAAAAAAAAAAAAAB shifted right once (the
// exact quotient by an invariant divisor, Granlund and Montgomery), the remainder M - 3 floor
// gives one more exact bit where the quotient is one bit short and a sticky bit, and the
// quotient is rounded to nearest even (x / 6 is never a midpoint: a midpoint times 6 would need
// more than 53 significant bits).  Valid for x zero or normal with 2^-1000 < |x| < 2^1000.
__device__ __forceinline__ double div6_x(double x) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned long long mg = u & 0x7fffffffffffffffULL;
  if (mg == 0) return x;  // +-0 / 6 = +-0
  const unsigned long long N = ((mg & 0xfffffffffffffULL) | 0x10000000000000ULL) << 11;
  const unsigned long long Q = __umul64hi(N, 0xAAAAAAAAAAAAAAABULL) >> 1;  // floor(N / 3)
  const unsigned long long R = N - 3ULL * Q;                                 // 0, 1 or 2
  unsigned long long V;
  long long e = (long long)(mg >> 52);
  if (Q >> 62) {  // leading 1 at bit 62
    V = Q;
    e -= 2;
  } else {        // at bit 61: append the next exact bit of N / 3
    V = 2ULL * Q + (R == 2ULL ? 1ULL : 0ULL);
    e -= 3;
  }
  unsigned long long m = V >> 10;
  const unsigned long long r = V & 0x3ffULL;
  if (r > 0x200ULL || (r == 0x200ULL && (R != 0ULL || (m & 1ULL)))) ++m;
  if (m >> 53) {
    m >>= 1;
    ++e;
  }
  return __longlong_as_double(
      (long long)((u & 0x8000000000000000ULL) | ((unsigned long long)e << 52) | (m & 0xfffffffffffffULL)));
}

// ---- IEEE double additions and small multiplications on the integer pipe ---------------
// Round-to-nearest-even sums and products by 3, 5/4 and 6 computed with 64-bit integer
// arithmetic (the textbook alignment with a sticky bit, guard bits, renormalisation and
// rounding), for operands that are zero or normal with 2^-900 < |x| < 2^900 and results that
// stay so -- every value the reconstruction forms from a tame window.  They return exactly the
// bits of the FP64 instruction they replace, on a pipe that retires ~60 times more lanes per
// clock than GB300's FP64 pipe.

// Pack a positive significand S (leading 1 at bit 62, sticky bits below bit 10) with biased
// exponent e and sign bit sg, rounding to nearest even.
__device__ __forceinline__ double round_pack_x(unsigned long long sg, long long e, unsigned long long S) {
  const unsigned long long r = S & 0x3ffULL;
  unsigned long long m = S >> 10;  // 53 bits, leading 1 at bit 52
  if (r > 0x200ULL || (r == 0x200ULL && (m & 1ULL))) ++m;
  if (m >> 53) {  // rounding carried into bit 53
    m >>= 1;
    ++e;
  }
  return __longlong_as_double((long long)(sg | ((unsigned long long)e << 52) | (m & 0xfffffffffffffULL)));
}

// RN(a + b)
__device__ __forceinline__ double add_x(double a, double b) {
  unsigned long long ua = (unsigned long long)__double_as_longlong(a);
  unsigned long long ub = (unsigned long long)__double_as_longlong(b);
  unsigned long long ma = ua & 0x7fffffffffffffffULL, mb = ub & 0x7fffffffffffffffULL;
  if (mb > ma) {  // |a| >= |b| from here on
    const unsigned long long t = ua;
    ua = ub;
    ub = t;
    const unsigned long long tm = ma;
    ma = mb;
    mb = tm;
  }
  const unsigned long long sg = ua & 0x8000000000000000ULL;
  if (mb == 0) {  // b is a zero: a, or the sum of two zeros (-0 only for -0 + -0)
    if (ma != 0) return __longlong_as_double((long long)ua);
    return __longlong_as_double((long long)(ua & ub));
  }
  const long long ea = (long long)(ma >> 52), eb = (long long)(mb >> 52);
  const long long d = ea - eb;
  if (d > 55) return __longlong_as_double((long long)ua);  // |b| below a quarter ulp of a
  // significands with 9 guard bits (leading 1 at bit 61); b's shifted out bits as a sticky bit
  const unsigned long long A = ((ma & 0xfffffffffffffULL) | 0x10000000000000ULL) << 9;
  const unsigned long long Bf = ((mb & 0xfffffffffffffULL) | 0x10000000000000ULL) << 9;
  const unsigned long long Bt = Bf >> d;
  const unsigned long long st = ((Bf << (63 - d)) << 1) != 0 ? 1ULL : 0ULL;  // only for d >= 10
  long long e = ea;
  unsigned long long S;
  if (((ua ^ ub) >> 63) == 0) {  // same signs: the sum's floor, sticky; leading 1 at bit 61 or 62
    S = (A + Bt) | st;
    if (S >> 62) {
      S = (S >> 1) | (S & 1ULL);
      ++e;
    }
    S <<= 1;  // leading 1 at bit 62
  } else {  // the difference's floor (sticky: b was truncated, subtract one more), then sticky
    S = A - Bt - st;
    if (S == 0) return 0.0;  // x - x = +0 (st is 0 then)
    const int sh = __clzll((long long)S) - 1;  // bring the leading 1 to bit 62 (sh <= 2 if st)
    S = (S << sh) | st;
    e -= sh - 1;
  }
  return round_pack_x(sg, e, S);
}
__device__ __forceinline__ double sub_x(double a, double b) {
  return add_x(a, __longlong_as_double(__double_as_longlong(b) ^ (long long)0x8000000000000000ULL));
}

// RN(k * x) for k = C * 2^S2 with a small odd integer C (3: k = 3 or 6; 5: k = 1.25)
template <int C, int S2>
__device__ __forceinline__ double mulk_x(double x) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned long long m = u & 0x7fffffffffffffffULL;
  if (m == 0) return x;  // k * +-0 = +-0
  const unsigned long long P = ((m & 0xfffffffffffffULL) | 0x10000000000000ULL) * (unsigned long long)C;
  const int sh = __clzll((long long)P) - 1;  // leading 1 to bit 62
  // P << sh holds the value's significand in bits 62..10: exponent field E + 10 + S2 - sh
  const long long e = (long long)(m >> 52) + 10 + S2 - sh;
  return round_pack_x(u & 0x8000000000000000ULL, e, P << sh);
}

// ---- gamma-dependent constants of a pack (fast mode) ---------------------------
struct GasConsts {
  double gm1, igm1, gamma;      // eos/gm1, 1/gm1, gm1+1
  double c2g;                   // C^2 * gamma
  double one_igm1;              // 1 + 1/gm1
  double hlle_k;                // (gamma+1)/sqrt(2 gamma)
  double hllc_k;                // (gamma+1)/(2 gamma)
};

// ---- ideal gas (singularity-eos IdealGas) ------------------------------------
__device__ __forceinline__ double eos_pressure(double gm1, double rho, double sie) {
  const double p = gm1 * rho * sie;
  return is_neg(p) ? 0.0 : p;
}
__device__ __forceinline__ double eos_bulk_modulus(double gm1, double rho, double sie) {
  const double small = 10.0 * 2.2250738585072014e-308;
  const double b = gm1 * (gm1 + 1.0) * rho * sie;
  return lt(small, b) ? b : small;
}

// RN(a / b) given y = RN(1 / b), by Markstein's theorem (P. W. Markstein, "Computation of
// elementary functions on the IBM RISC System/6000 processor", IBM J. Res. Develop. 34(1),
// 1990, Theorem 1): q = RN(a y) lies within one ulp of a / b, so the remainder a - b q is
// exact (one fused multiply-add), and RN(q + (a - b q) y) is the correctly rounded quotient.
// For a and b tame (b nonzero), where no product or remainder leaves the normal range; a zero
// remainder means q = a / b exactly (and keeps the sign of a zero quotient).
__device__ __forceinline__ double div_rcp(double a, double b, double y) {
  const double q = __dmul_rn(a, y);
  if ((((unsigned)__double2hiint(a) & 0x7fffffffu) | (unsigned)__double2loint(a)) == 0u) return q;
  return __fma_rn(__fma_rn(-q, b, a), y, q);  // a nonzero: q nonzero, and q + (+-0) == q
}

// a / b correctly rounded, from y = RN(1 / b) where a and b allow it (the division otherwise).
__device__ __forceinline__ double div_y(double a, double b, double y) {
  return (tame(a) && tame_nz(b)) ? div_rcp(a, b, y) : a / b;
}

// a1 / b and a2 / b correctly rounded, sharing one reciprocal where the operands allow.
__device__ __forceinline__ void div2(double a1, double a2, double b, double &q1, double &q2) {
  if (tame(a1) && tame(a2) && tame_nz(b)) {
    const double y = __drcp_rn(b);
    q1 = div_rcp(a1, b, y);
    q2 = div_rcp(a2, b, y);
  } else {
    q1 = a1 / b;
    q2 = a2 / b;
  }
}

// The reference's ConsToPrim arithmetic after the density floor (hydro.cpp:502-531), one
// rounded operation at a time in its order: the fast build contracts products and sums into
// FMAs, and these values must match the reference bit for bit where they feed the
// discontinuous PPM limiters (the adiabatic-index fields of blocks where a floor fired, which
// the fast mode otherwise replaces by the constants) or the non-idempotent pressure floor.
// u_d: the floored density, di = 1 / u_d.  Sets u[IEN], w[IPR], g_c, g_e; returns whether
// the pressure floor fired.
__device__ __forceinline__ bool cons_to_prim_tail(double *u, double *w, double &g_c, double &g_e,
                                                  double u_d, double di, double gm1, double pfloor) {
  const double m1 = u[IM1], m2 = u[IM2], m3 = u[IM3];
  const double e_k = __dmul_rn(__dmul_rn(0.5, di),
                               __dadd_rn(__dadd_rn(__dmul_rn(m1, m1), __dmul_rn(m2, m2)), __dmul_rn(m3, m3)));
  double u_e = u[IEN];
  double sie = div_y(__dsub_rn(u_e, e_k), u_d, di);  // (u_e - e_k) / u_d
  double w_p = __dmul_rn(__dmul_rn(gm1, u_d), sie);
  w_p = is_neg(w_p) ? 0.0 : w_p;  // eos_pressure
  const bool floored = !gt(w_p, pfloor);
  if (floored) {
    const double gm1q = __ddiv_rn(w_p, __dmul_rn(u_d, e_k));  // hydro.cpp:517
    u_e = __dadd_rn(__ddiv_rn(pfloor, gm1q), e_k);
    w_p = pfloor;
    sie = div_y(__dsub_rn(u_e, e_k), u_d, di);  // of the floored energy (unchanged otherwise)
  }
  u[IEN] = u_e;
  w[IPR] = w_p;
  const double small = 10.0 * 2.2250738585072014e-308;
  double b = __dmul_rn(__dmul_rn(__dmul_rn(gm1, __dadd_rn(gm1, 1.0)), u_d), sie);  // eos_bulk_modulus
  b = lt(small, b) ? b : small;
  g_c = __ddiv_rn(b, w_p);
  g_e = __dadd_rn(__ddiv_rn(w_p, __dsub_rn(u_e, e_k)), 1.0);
  return floored;
}

// ConsToPrim for one cell (hydro.cpp:459-531, ideal gas).  u[] is updated in place
// by the floors (density, energy); w[] gets rho, v1, v2, v3, p; g_c, g_e the two
// adiabatic indices.  Returns true when the pressure floor was applied.
__device__ __forceinline__ bool cons_to_prim_cell(double *u, double *w, double &g_c, double &g_e,
                                                  double gm1, double dfloor, double pfloor) {
  double u_d = u[IDN];
  const bool dens_ok = gt(u_d, dfloor);
  u_d = dens_ok ? u_d : dfloor;
  u[IDN] = u_d;
  const double di = __drcp_rn(u_d);  // the correctly rounded 1.0 / u_d
  w[IDN] = u_d;
  w[IV1] = u[IM1] * di;
  w[IV2] = u[IM2] * di;
  w[IV3] = u[IM3] * di;
#if !APH_EXACT
  // fast: p = gm1 rho ((E - e_k) / rho) = gm1 (E - e_k), and with the floors inactive both
  // adiabatic indices are gamma (B / p = gm1 + 1 = p / (rho e) + 1), so one division per cell
  // (a floored density takes the reference's arithmetic below, whose indices are kept)
  if (dens_ok) {
    const double e_k = 0.5 * di * (u[IM1] * u[IM1] + u[IM2] * u[IM2] + u[IM3] * u[IM3]);
    const double pe = gm1 * (u[IEN] - e_k);
    const double wp = is_neg(pe) ? 0.0 : pe;
    if (gt(wp, pfloor)) {
      w[IPR] = wp;
      g_c = gm1 + 1.0;
      g_e = g_c;
      return false;
    }
  }
#endif
  return cons_to_prim_tail(u, w, g_c, g_e, u_d, di, gm1, pfloor);
}

// The reference's adiabatic indices (gamma_c, gamma_e) of a cell whose floors did not fire,
// from its conserved state after ConsToPrim (u: the cell's five values).
__device__ __forceinline__ void gamma_ref(const double *u, double gm1, double &g_c, double &g_e) {
  double uu[NHYDRO] = {u[0], u[1], u[2], u[3], u[4]}, w[NHYDRO];
  cons_to_prim_tail(uu, w, g_c, g_e, u[IDN], 1.0 / u[IDN], gm1, -1.0);
}

// ---- reconstruction (src/recon) --------------------------------------------------
__device__ __forceinline__ void plm(double q_im1, double q_i, double q_ip1, double &ql_ip1,
                                    double &qr_i) {
  const double dql = q_i - q_im1;
  const double dqr = q_ip1 - q_i;
  const double dq2 = dql * dqr;
  double dqm = 0.0;
  if (is_pos(dq2)) dqm = dq2 / (dql + dqr);
  ql_ip1 = q_i + dqm;
  qr_i = q_i - dqm;
}

// PPM split in two.  The limited interface value at a face is a function of the four
// cells around it only, and the reference computes it identically from both adjacent
// cells (its symmetric grouping of the stencil sums makes the two evaluations the same
// operations on the same operands).  ppm_face() evaluates it once per face;
// ppm_cell() then applies the cell's parabola limiter.  Together they give exactly
// PPM(q_im2..q_ip2) of ppm_simple.hpp:32-161.
//
// dd(c) = 0.5*(q[c+1]-q[c]) + 0.5*(q[c]-q[c-1]);  d2(c) = (q[c-1]+q[c+1]) - 2*q[c]
//
// TAME (exact mode, every window value tame): the same bits with the scalings by 2, 1/2
// and 1/6 and the sign tests of products of differences on the integer pipe.
template <bool TAME = false>
__device__ __forceinline__ double ppm_dd(double qm1, double q0, double qp1) {
#if APH_EXACT
  if (TAME) return add_x(half_x(sub_x(qp1, q0)), half_x(sub_x(q0, qm1)));
  return 0.5 * (qp1 - q0) + 0.5 * (q0 - qm1);
#else
  return 0.5 * (qp1 - qm1);  // the same quantity with one rounding
#endif
}
template <bool TAME = false>
__device__ __forceinline__ double ppm_d2(double qm1, double q0, double qp1) {
  if (APH_EXACT && TAME) return sub_x(add_x(qm1, qp1), twice_x(q0));
  return (qm1 + qp1) - 2.0 * q0;
}
// Face between cells c-1 (value qm1) and c (value q0): ddm1 = dd(c-1), dd0 = dd(c),
// d2m1 = d2(c-1), d20 = d2(c).
template <bool TAME = false>
__device__ __forceinline__ double ppm_face(double qm1, double q0, double ddm1, double dd0,
                                           double d2m1, double d20) {
#if APH_EXACT
  if (TAME) {
    const double s = add_x(qm1, q0);  // the additions and the x3, x5/4 scalings on the integer pipe
    const double avg = half_x(s);
    double dph = add_x(avg, div6_x(sub_x(ddm1, dd0)));
    const double qa = mulk_x<3, 0>(sub_x(s, twice_x(dph)));
    double qd = 0.0;
    const bool sa = is_neg(qa);
    if (sa == is_neg(d2m1) && sa == is_neg(d20)) {
      const unsigned long long mb = mag(d2m1), mc = mag(d20);
      const double m = mulk_x<5, -2>(from_bits(mc < mb ? mc : mb));  // PPM_C2 = 5/4
      const unsigned long long mm = mag(m), ma = mag(qa);
      qd = flip_if(from_bits(ma < mm ? ma : mm), sa);
    }
    // (dph - qm1) * (q0 - dph) < 0, the differences being nonzero and their product normal
    if (strictly_outside(dph, qm1, q0)) dph = sub_x(avg, div6_x(qd));
    return dph;
  }
#endif
  const double avg = 0.5 * (qm1 + q0);
#if APH_EXACT
  double dph = avg + (ddm1 - dd0) / 6.0;
#else
  double dph = fma(ddm1 - dd0, 1.0 / 6.0, avg);
#endif
#if APH_EXACT
  const double qa_tmp = dph - qm1;
  const double qb_tmp = q0 - dph;
#endif
  const double qa = 3.0 * (qm1 + q0 - 2.0 * dph);
  double qd = 0.0;
  const bool sa = is_neg(qa);
  if (sa == is_neg(d2m1) && sa == is_neg(d20)) {
    // min(C2|qb|, min(C2|qc|, |qa|)) with the two scalings merged (scaling by a positive
    // constant is monotone, so min(C2 x, C2 y) == C2 min(x, y) bit for bit)
    const unsigned long long mb = mag(d2m1), mc = mag(d20);
    const double m = PPM_C2 * from_bits(mc < mb ? mc : mb);
    const unsigned long long mm = mag(m), ma = mag(qa);
    qd = flip_if(from_bits(ma < mm ? ma : mm), sa);
  }
#if APH_EXACT
  if (is_neg(qa_tmp * qb_tmp)) dph = avg - qd / 6.0;
#else
  if (strictly_outside(dph, qm1, q0)) dph = fma(qd, -1.0 / 6.0, avg);
#endif
  return dph;
}

// Cell limiter: dph_lo, dph_hi are the limited values at faces i-1/2, i+1/2.
// Outputs ql_ip1 (left state of face i+1/2) and qr_i (right state of face i-1/2).
template <bool TAME = false>
__device__ __forceinline__ void ppm_cell(double q_im2, double q_im1, double q_i, double q_ip1,
                                         double q_ip2, double d2m1, double d20, double d2p1,
                                         double dph_lo, double dph_hi, double &ql_ip1,
                                         double &qr_i) {
  constexpr bool T = APH_EXACT && TAME;
  const double d2qf = T ? mulk_x<3, 1>(sub_x(add_x(dph_lo, dph_hi), twice_x(q_i)))
                        : 6.0 * (dph_lo + dph_hi - 2.0 * q_i);
  double qr = dph_lo, ql = dph_hi;
  const double dqf_minus = T ? sub_x(q_i, qr) : q_i - qr;
  const double dqf_plus = T ? sub_x(ql, q_i) : ql - q_i;
#if APH_EXACT
  bool extremum;
  if (T) {  // the two products' signs, as in ppm_face
    extremum = !strictly_between(qr, q_i, ql) || !strictly_between(q_im1, q_i, q_ip1);
  } else {
    const double qa_tmp = dqf_minus * dqf_plus;
    const double qb_tmp = (q_ip1 - q_i) * (q_i - q_im1);
    extremum = !is_pos(qa_tmp) || !is_pos(qb_tmp);
  }
  if (extremum) {
#else
  if (!strictly_between(qr, q_i, ql) || !strictly_between(q_im1, q_i, q_ip1)) {
#endif
    // local extremum: limit with rho = qe/qd (CS eq 22-23, MC eq 27)
    double qe = 0.0;
    const bool sd = is_neg(d2qf);
    if (sd == is_neg(d2m1) && sd == is_neg(d20) && sd == is_neg(d2p1)) {
      unsigned long long m = mag(d2m1);
      const unsigned long long m0 = mag(d20), m1 = mag(d2p1);
      m = m0 < m ? m0 : m;
      m = m1 < m ? m1 : m;
      const unsigned long long ms = mag(T ? mulk_x<5, -2>(from_bits(m)) : PPM_C2 * from_bits(m));
      const unsigned long long md = mag(d2qf);
      qe = flip_if(from_bits(md < ms ? md : ms), sd);
    }
    unsigned long long mx = mag(q_im2);
    const unsigned long long a1 = mag(q_im1), a2 = mag(q_i), a3 = mag(q_ip1), a4 = mag(q_ip2);
    mx = a1 > mx ? a1 : mx;
    mx = a2 > mx ? a2 : mx;
    mx = a3 > mx ? a3 : mx;
    mx = a4 > mx ? a4 : mx;
    double rho = 0.0;
    // the roundoff guard |d2qf| > 1e-12 * max|q| (ppm_simple.hpp:132); RN(1e-12 * mx) lies in
    // [2^-40, 2^-38) times mx's binade, so the exponents decide it except within two binades
    bool guard;
    if (T) {
      const long long ed = (long long)(mag(d2qf) >> 52), em = (long long)(mx >> 52);
      if (mag(d2qf) == 0) guard = false;  // 0 > anything is false
      else if (mx == 0) guard = true;      // a nonzero value over 1e-12 * 0
      else if (ed >= em - 38) guard = true;
      else if (ed <= em - 41) guard = false;
      else guard = mag(d2qf) > mag(1.0e-12 * from_bits(mx));
    } else {
      guard = mag(d2qf) > mag(1.0e-12 * from_bits(mx));
    }
#if APH_EXACT
    if (T && ((__double_as_longlong(qe) << 1) == 0 || !guard)) {
      // rho is a zero (+0 without the guard, else qe / d2qf = +-0 by the signs): the products
      // rho * dqf are zeros with the product of the signs, and no division is needed
      const long long rs = guard ? ((__double_as_longlong(qe) ^ __double_as_longlong(d2qf)) &
                                    (long long)0x8000000000000000ULL) : 0LL;
      const double zm = __longlong_as_double(rs ^ (__double_as_longlong(dqf_minus) & (long long)0x8000000000000000ULL));
      const double zp = __longlong_as_double(rs ^ (__double_as_longlong(dqf_plus) & (long long)0x8000000000000000ULL));
      qr = sub_x(q_i, zm);
      ql = add_x(q_i, zp);
    } else if (T && __double_as_longlong(qe) == __double_as_longlong(d2qf)) {
      // rho = d2qf / d2qf = 1 > 1 - 1e-12: the face values stay
    } else {
      if (guard) rho = qe / d2qf;
      if (le(rho, 1.0 - 1.0e-12)) {
        qr = T ? sub_x(q_i, rho * dqf_minus) : q_i - rho * dqf_minus;
        ql = T ? add_x(q_i, rho * dqf_plus) : q_i + rho * dqf_plus;
      }
    }
#else
    if (guard) rho = qe / d2qf;
    if (le(rho, 1.0 - 1.0e-12)) {
      qr = fma(-rho, dqf_minus, q_i);
      ql = fma(rho, dqf_plus, q_i);
    }
#endif
  } else {
    if (mag(dqf_minus) >= twice_mag(dqf_plus))
      qr = T ? sub_x(q_i, twice_x(dqf_plus)) : q_i - 2.0 * dqf_plus;
    if (mag(dqf_plus) >= twice_mag(dqf_minus))
      ql = T ? add_x(q_i, twice_x(dqf_minus)) : q_i + 2.0 * dqf_minus;
  }
  ql_ip1 = ql;
  qr_i = qr;
}

// Whole-cell PPM from the five-point stencil (used where the face values are not shared).
__device__ __forceinline__ void ppm(double q_im2, double q_im1, double q_i, double q_ip1,
                                    double q_ip2, double &ql_ip1, double &qr_i) {
  const double dd_m1 = ppm_dd(q_im2, q_im1, q_i);
  const double dd_0 = ppm_dd(q_im1, q_i, q_ip1);
  const double dd_p1 = ppm_dd(q_i, q_ip1, q_ip2);
  const double d2_m1 = ppm_d2(q_im2, q_im1, q_i);
  const double d2_0 = ppm_d2(q_im1, q_i, q_ip1);
  const double d2_p1 = ppm_d2(q_i, q_ip1, q_ip2);
  const double lo = ppm_face(q_im1, q_i, dd_m1, dd_0, d2_m1, d2_0);
  const double hi = ppm_face(q_i, q_ip1, dd_0, dd_p1, d2_0, d2_p1);
  ppm_cell(q_im2, q_im1, q_i, q_ip1, q_ip2, d2_m1, d2_0, d2_p1, lo, hi, ql_ip1, qr_i);
}

template <int RECON>
__device__ __forceinline__ void reconstruct(const double *q, double &ql_ip1, double &qr_i) {
  // q[-2..2] addressable around q[0]
  if (RECON == RECON_DC) {
    ql_ip1 = qr_i = q[0];
  } else if (RECON == RECON_PLM) {
    plm(q[-1], q[0], q[1], ql_ip1, qr_i);
  } else {
    ppm(q[-2], q[-1], q[0], q[1], q[2], ql_ip1, qr_i);
  }
}

// ---- Riemann solvers (src/hydro/rsolvers) -------------------------------------------
// wl, wr: (rho, v_normal, v_t1, v_t2, p).  gl*, gr*: reconstructed (gamma_c, gamma_e).
// With CONSTG the adiabatic indices are the pack's constants (gc) instead.
// flx: (mass, normal momentum, t1 momentum, t2 momentum, energy).

// c-limited sound speed C*sqrt(gamma / (1 + (1/gm1 + rho C^2 / p))) (hydro_hlle.hpp:63-66)
template <bool CONSTG>
__device__ __forceinline__ double sound_speed(double rho, double p, double gamma, double igm1,
                                              const GasConsts &gc) {
#if APH_EXACT
  return C_LIGHT * sqrt(gamma / (1 + (igm1 + rho * C_LIGHT2 / p)));
#else
  // same quantity as sqrt(C^2 gamma p / (p (1 + 1/gm1) + rho C^2))
  const double num = (CONSTG ? gc.c2g : C_LIGHT2 * gamma) * p;
  const double den = fma(p, CONSTG ? gc.one_igm1 : 1.0 + igm1, rho * C_LIGHT2);
  return num * rsqrt(num * den);
#endif
}

template <bool CONSTG>
__device__ __forceinline__ void solve_hlle(const double *wli, const double *wri, double glc,
                                           double gle, double grc, double gre,
                                           const GasConsts &gc, double *flxi) {
  const double gammal = CONSTG ? gc.gamma : glc;
  const double gammar = CONSTG ? gc.gamma : grc;
  double igm1l, igm1r;
  if (CONSTG) {
    igm1l = igm1r = gc.igm1;
  } else {
    igm1l = __drcp_rn(gle - 1);  // the correctly rounded 1.0 / (gle - 1), cheaper than a division
    igm1r = __drcp_rn(gre - 1);
  }
  const double cl = sound_speed<CONSTG>(wli[IDN], wli[IPR], gammal, igm1l, gc);
  const double cr = sound_speed<CONSTG>(wri[IDN], wri[IPR], gammar, igm1r, gc);
  const double el = wli[IPR] * igm1l +
                    0.5 * wli[IDN] * (wli[IV1] * wli[IV1] + wli[IV2] * wli[IV2] + wli[IV3] * wli[IV3]);
  const double er = wri[IPR] * igm1r +
                    0.5 * wri[IDN] * (wri[IV1] * wri[IV1] + wri[IV2] * wri[IV2] + wri[IV3] * wri[IV3]);
  const double rhoa = .5 * (wli[IDN] + wri[IDN]);
  const double ca = .5 * (cl + cr);
  const double pmid = .5 * (wli[IPR] + wri[IPR] + (wli[IV1] - wri[IV1]) * rhoa * ca);
  double ql = 1.0, qr = 1.0;
#if APH_EXACT
  if (gt(pmid, wli[IPR])) ql = 1.0 + (gammal + 1) / sqrt(2 * gammal) * (pmid / wli[IPR] - 1.0);
  if (gt(pmid, wri[IPR])) qr = 1.0 + (gammar + 1) / sqrt(2 * gammar) * (pmid / wri[IPR] - 1.0);
#else
  {
    const bool bl = gt(pmid, wli[IPR]), br = gt(pmid, wri[IPR]);
    if (bl || br) {
      const double ipp = 1.0 / (wli[IPR] * wri[IPR]);  // shared reciprocal
      const double kl = CONSTG ? gc.hlle_k : (gammal + 1) * rsqrt(2 * gammal);
      const double kr = CONSTG ? gc.hlle_k : (gammar + 1) * rsqrt(2 * gammar);
      if (bl) ql = fma(kl, fma(pmid * wri[IPR], ipp, -1.0), 1.0);
      if (br) qr = fma(kr, fma(pmid * wli[IPR], ipp, -1.0), 1.0);
    }
  }
#endif
  const double al = wli[IV1] - cl * ql;
  const double ar = wri[IV1] + cr * qr;
  const double bp = is_pos(ar) ? ar : 0.0;
  const double bm = is_neg(al) ? al : 0.0;
  const double vxl = wli[IV1] - bm;
  const double vxr = wri[IV1] - bp;
  double fl[NHYDRO], fr[NHYDRO];
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
  double tmp = 0.0;
  if (__double_as_longlong(bp) != __double_as_longlong(bm) && (mag(bp) | mag(bm)) != 0ULL)
    tmp = 0.5 * (bp + bm) / (bp - bm);
#pragma unroll
  for (int n = 0; n < NHYDRO; ++n) flxi[n] = 0.5 * (fl[n] + fr[n]) + (fl[n] - fr[n]) * tmp;
}

// x = 2^k with x and 1/x both normal: then y / x == y * (1/x) exactly for every y (both are
// the correctly rounded y * 2^-k), so a division by x is a multiplication.
__device__ __forceinline__ bool pow2_normal(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned long long e = b >> 52;  // the sign bit must be 0
  return (b & 0xfffffffffffffULL) == 0 && e >= 1 && e <= 2045;
}
// y / vol, correctly rounded; ivol = 1 / vol, p2 = pow2_normal(vol) (uniform over a block)
__device__ __forceinline__ double div_vol(double y, double vol, double ivol, bool p2) {
  if (p2) return y * ivol;
  return y / vol;
}

// The reference's c-limited sound speed C sqrt(gamma / (1 + (igm1 + rho C^2 / p)))
// (hydro_hllc.hpp:57-60) with its roundings.  Where X = rho C^2 / p is at least 2^55 times
// both igm1 and 1 (always for non-relativistic gas: X ~ (c_light / c_sound)^2), each addition
// adds less than a quarter ulp of X and returns X, so both are skipped.
__device__ __forceinline__ double csound_exact(double rho, double p, double gamma, double igm1, double yp) {
  const double X = div_y(rho * C_LIGHT2, p, yp);
  const long long ex = (long long)(mag(X) >> 52), ei = (long long)(mag(igm1) >> 52);
  const double den = (ex >= 1023 + 55 && ex >= ei + 55 && ex < 2047) ? X : 1 + (igm1 + X);
  return C_LIGHT * sqrt(gamma / den);
}

// exponent field all ones: an infinity or a NaN
__device__ __forceinline__ bool nonfinite(double x) {
  return ((__double2hiint(x) >> 20) & 0x7ff) == 0x7ff;
}

// HLLC in the exact mode with the reference's roundings (hydro_hllc.hpp:45-145, and the
// low-Mach pstar of hydro_lhllc.hpp:71-79), arranged for the GPU without changing a bit:
//  * the shock factor (gamma_l + 1) / (2 gamma_r), which the reference writes identically
//    for both sides, is formed once, and a face shocked on one side only takes one
//    division and square root whichever side it is;
//  * the contact branch picks its operands instead of its code, so both branches are the
//    same two divisions: ul = sstar / (sstar - bm), ustar = -bm / (sstar - bm) when
//    sstar >= 0, else ur = -sstar / (bp - sstar), ustar = bp / (bp - sstar);
//  * TAME (the reconstruction window was tame): the flux is formed from the upwind side only.
//    The reference's ul*fl + ur*fr has one weight exactly 0, and RN(a + (+-0)) == a for a
//    nonzero a, so the other side's term (0 * f, a signed zero: no product of values derived
//    from a tame window overflows) is added, in the reference's order, only where the upwind
//    term is zero and the sign of the zero sum depends on it, or where the other side is
//    not finite.  The halvings and doublings run on the integer pipe (half_x, twice_x).
//    Without TAME both sides' terms are always formed.
template <bool LOWMACH, bool TAME>
__device__ __forceinline__ void solve_hllc_exact(const double *wli, const double *wri, double glc,
                                                 double gle, double grc, double gre, double *flxi) {
  auto hlf = [](double x) { return TAME ? half_x(x) : 0.5 * x; };
  const double gammal = glc, gammar = grc;
  const double igm1l = __drcp_rn(gle - 1), igm1r = __drcp_rn(gre - 1);  // == 1.0 / (g - 1)
  // 1 / p of each side: the sound speed and the shock factor divide by p (div_y; unused
  // where the operands leave the tame range and the divisions are made as such)
  const double ypl = __drcp_rn(wli[IPR]), ypr = __drcp_rn(wri[IPR]);
  const double cl = csound_exact(wli[IDN], wli[IPR], gammal, igm1l, ypl);
  const double cr = csound_exact(wri[IDN], wri[IPR], gammar, igm1r, ypr);
  const double rhoa = hlf(wli[IDN] + wri[IDN]);
  const double ca = hlf(cl + cr);
  double pstar;
  if (!LOWMACH) {
    pstar = hlf(wli[IPR] + wri[IPR]) - hlf(wri[IV1] - wli[IV1]) * rhoa * ca;
  } else {
    const double machl = sqrt(wli[IV1] * wli[IV1] + wli[IV2] * wli[IV2] + wli[IV3] * wli[IV3]);
    const double machr = sqrt(wri[IV1] * wri[IV1] + wri[IV2] * wri[IV2] + wri[IV3] * wri[IV3]);
    const double chi = smax(machl, machr);
    const double phi = chi * (2.0 - chi);
    pstar = hlf(wli[IPR] + wri[IPR]) - hlf(wri[IV1] - wli[IV1]) * rhoa * ca * phi;
  }
  double ql = 1.0, qr = 1.0;
  const bool bl = gt(pstar, wli[IPR]), br = gt(pstar, wri[IPR]);
  if (bl || br) {
    const double k = (gammal + 1) / (TAME ? twice_x(gammar) : 2 * gammar);
    const double q1 = sqrt(1.0 + k * (div_y(pstar, bl ? wli[IPR] : wri[IPR], bl ? ypl : ypr) - 1.0));
    if (bl) ql = q1;
    else qr = q1;
    if (bl && br) qr = sqrt(1.0 + k * (div_y(pstar, wri[IPR], ypr) - 1.0));
  }
  const double sl = wli[IV1] - cl * ql;
  const double sr = wri[IV1] + cr * qr;
  const double bp = is_pos(sr) ? sr : TINY_NUMBER;
  const double bm = is_neg(sl) ? sl : -TINY_NUMBER;
  const double vxl0 = wli[IV1] - sl;
  const double vxr0 = wri[IV1] - sr;
  const double tl = wli[IPR] + vxl0 * wli[IDN] * wli[IV1];
  const double tr = wri[IPR] + vxr0 * wri[IDN] * wri[IV1];
  const double ml = wli[IDN] * vxl0;
  const double mr = -(wri[IDN] * vxr0);
  double sstar, cp;  // (tl - tr) / (ml + mr), (ml tr + mr tl) / (ml + mr)
  div2(tl - tr, ml * tr + mr * tl, ml + mr, sstar, cp);
  cp = is_pos(cp) ? cp : 0.0;
  const bool L = !is_neg(sstar);  // sstar >= 0.0
  const double den = L ? sstar - bm : bp - sstar;
  double coef, ustar;  // ul (or ur) and ustar: (+-sstar) / den, (-bm or bp) / den
  div2(L ? sstar : -sstar, L ? -bm : bp, den, coef, ustar);
  // the upwind side (U) and the other one (O)
  const double *wu = L ? wli : wri, *wo = L ? wri : wli;
  const double igu = L ? igm1l : igm1r;
  const double bu = L ? bm : bp, bo = L ? bp : bm;
  const double vx = wu[IV1] - bu;
  double f[NHYDRO];
  f[IDN] = wu[IDN] * vx;
  f[IV1] = wu[IDN] * wu[IV1] * vx + wu[IPR];
  f[IV2] = wu[IDN] * wu[IV2] * vx;
  f[IV3] = wu[IDN] * wu[IV3] * vx;
  const double eu = wu[IPR] * igu + hlf(wu[IDN]) * (wu[IV1] * wu[IV1] + wu[IV2] * wu[IV2] + wu[IV3] * wu[IV3]);
  f[IEN] = eu * vx + wu[IPR] * wu[IV1];
  const bool obad = nonfinite(wo[IDN]) || nonfinite(wo[IV1]) || nonfinite(wo[IV2]) ||
                    nonfinite(wo[IV3]) || nonfinite(wo[IPR]) || nonfinite(bo) ||
                    nonfinite(L ? igm1r : igm1l);
  double t[NHYDRO];
#pragma unroll
  for (int n = 0; n < NHYDRO; ++n) {
    t[n] = coef * f[n];
    if (!TAME || obad || (__double_as_longlong(t[n]) << 1) == 0) {  // add the reference's 0 * fo
      const double vxo = wo[IV1] - bo;
      double fo;
      if (n == IDN) fo = wo[IDN] * vxo;
      else if (n == IV1) fo = wo[IDN] * wo[IV1] * vxo + wo[IPR];
      else if (n == IV2) fo = wo[IDN] * wo[IV2] * vxo;
      else if (n == IV3) fo = wo[IDN] * wo[IV3] * vxo;
      else {
        const double eo = wo[IPR] * (L ? igm1r : igm1l) +
                          hlf(wo[IDN]) * (wo[IV1] * wo[IV1] + wo[IV2] * wo[IV2] + wo[IV3] * wo[IV3]);
        fo = eo * vxo + wo[IPR] * wo[IV1];
      }
      const double zo = 0.0 * fo;
      t[n] = L ? t[n] + zo : zo + t[n];  // the reference's order: ul*fl + ur*fr
    }
  }
  flxi[IDN] = t[IDN];
  flxi[IV1] = t[IV1] + ustar * cp;
  flxi[IV2] = t[IV2];
  flxi[IV3] = t[IV3];
  flxi[IEN] = t[IEN] + ustar * cp * sstar;
}

template <bool CONSTG, bool LOWMACH>
__device__ __forceinline__ void solve_hllc(const double *wli, const double *wri, double glc,
                                           double gle, double grc, double gre,
                                           const GasConsts &gc, double *flxi) {
  const double gammal = CONSTG ? gc.gamma : glc;
  const double gammar = CONSTG ? gc.gamma : grc;
  double igm1l, igm1r;
  if (CONSTG) {
    igm1l = igm1r = gc.igm1;
  } else {
    igm1l = __drcp_rn(gle - 1);  // the correctly rounded 1.0 / (gle - 1), cheaper than a division
    igm1r = __drcp_rn(gre - 1);
  }
  const double cl = sound_speed<CONSTG>(wli[IDN], wli[IPR], gammal, igm1l, gc);
  const double cr = sound_speed<CONSTG>(wri[IDN], wri[IPR], gammar, igm1r, gc);
  const double el = wli[IPR] * igm1l +
                    0.5 * wli[IDN] * (wli[IV1] * wli[IV1] + wli[IV2] * wli[IV2] + wli[IV3] * wli[IV3]);
  const double er = wri[IPR] * igm1r +
                    0.5 * wri[IDN] * (wri[IV1] * wri[IV1] + wri[IV2] * wri[IV2] + wri[IV3] * wri[IV3]);
  const double rhoa = .5 * (wli[IDN] + wri[IDN]);
  const double ca = .5 * (cl + cr);
  double pstar;
  if (!LOWMACH) {
    pstar = .5 * (wli[IPR] + wri[IPR]) - .5 * (wri[IV1] - wli[IV1]) * rhoa * ca;
  } else {
    // hydro_lhllc.hpp:71-79: "Mach" is the speed |v| itself
    const double machl = sqrt(wli[IV1] * wli[IV1] + wli[IV2] * wli[IV2] + wli[IV3] * wli[IV3]);
    const double machr = sqrt(wri[IV1] * wri[IV1] + wri[IV2] * wri[IV2] + wri[IV3] * wri[IV3]);
    const double chi = smax(machl, machr);
    const double phi = chi * (2.0 - chi);
    pstar = .5 * (wli[IPR] + wri[IPR]) - .5 * (wri[IV1] - wli[IV1]) * rhoa * ca * phi;
  }
  double ql = 1.0, qr = 1.0;
#if APH_EXACT
  if (gt(pstar, wli[IPR])) ql = sqrt(1.0 + (gammal + 1) / (2 * gammar) * (pstar / wli[IPR] - 1.0));
  if (gt(pstar, wri[IPR])) qr = sqrt(1.0 + (gammal + 1) / (2 * gammar) * (pstar / wri[IPR] - 1.0));
#else
  {
    const bool bl = gt(pstar, wli[IPR]), br = gt(pstar, wri[IPR]);
    if (bl || br) {
      const double ipp = 1.0 / (wli[IPR] * wri[IPR]);
      const double k = CONSTG ? gc.hllc_k : (gammal + 1) / (2 * gammar);
      if (bl) ql = sqrt(fma(k, fma(pstar * wri[IPR], ipp, -1.0), 1.0));
      if (br) qr = sqrt(fma(k, fma(pstar * wli[IPR], ipp, -1.0), 1.0));
    }
  }
#endif
  const double sl = wli[IV1] - cl * ql;
  const double sr = wri[IV1] + cr * qr;
  const double bp = is_pos(sr) ? sr : TINY_NUMBER;
  const double bm = is_neg(sl) ? sl : -TINY_NUMBER;
  double vxl = wli[IV1] - sl;
  double vxr = wri[IV1] - sr;
  const double tl = wli[IPR] + vxl * wli[IDN] * wli[IV1];
  const double tr = wri[IPR] + vxr * wri[IDN] * wri[IV1];
  const double ml = wli[IDN] * vxl;
  const double mr = -(wri[IDN] * vxr);
#if APH_EXACT
  const double sstar = (tl - tr) / (ml + mr);
  double cp = (ml * tr + mr * tl) / (ml + mr);
#else
  const double imm = 1.0 / (ml + mr);
  const double sstar = (tl - tr) * imm;
  double cp = (ml * tr + mr * tl) * imm;
#endif
  cp = is_pos(cp) ? cp : 0.0;
#if !APH_EXACT
  {
    // one-sided: the flux is sstar/(sstar - b) times the physical flux of the upwind side of
    // the contact (left with b = bm when sstar >= 0, else right with b = bp) plus the
    // pressure terms; the other side's weight is exactly 0, so this is the two-sided sum of
    // the reference with its zero term dropped
    const bool L = !is_neg(sstar);
    const double rho = L ? wli[IDN] : wri[IDN], u = L ? wli[IV1] : wri[IV1];
    const double v = L ? wli[IV2] : wri[IV2], z = L ? wli[IV3] : wri[IV3];
    const double p = L ? wli[IPR] : wri[IPR];
    const double b = L ? bm : bp;
    const double e = p * (L ? igm1l : igm1r) + 0.5 * rho * (u * u + v * v + z * z);
    const double id = 1.0 / (sstar - b);
    const double coef = sstar * id;
    const double ustar = -b * id;
    const double vx = u - b;
    flxi[IDN] = coef * (rho * vx);
    flxi[IV1] = coef * (rho * u * vx + p) + ustar * cp;
    flxi[IV2] = coef * (rho * v * vx);
    flxi[IV3] = coef * (rho * z * vx);
    flxi[IEN] = coef * (e * vx + p * u) + ustar * cp * sstar;
    return;
  }
#endif
  vxl = wli[IV1] - bm;
  vxr = wri[IV1] - bp;
  double fl[NHYDRO], fr[NHYDRO];
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
  double ul, ur, ustar;
  if (!is_neg(sstar)) {  // sstar >= 0.0
#if APH_EXACT
    ul = sstar / (sstar - bm);
    ustar = -bm / (sstar - bm);
#else
    const double id = 1.0 / (sstar - bm);
    ul = sstar * id;
    ustar = -bm * id;
#endif
    ur = 0.0;
  } else {
#if APH_EXACT
    ur = -sstar / (bp - sstar);
    ustar = bp / (bp - sstar);
#else
    const double id = 1.0 / (bp - sstar);
    ur = -sstar * id;
    ustar = bp * id;
#endif
    ul = 0.0;
  }
  flxi[IDN] = ul * fl[IDN] + ur * fr[IDN];
  flxi[IV1] = ul * fl[IV1] + ur * fr[IV1] + ustar * cp;
  flxi[IV2] = ul * fl[IV2] + ur * fr[IV2];
  flxi[IV3] = ul * fl[IV3] + ur * fr[IV3];
  flxi[IEN] = ul * fl[IEN] + ur * fr[IEN] + ustar * cp * sstar;
}

template <int RS, bool CONSTG, bool TAME = false>
__device__ __forceinline__ void riemann(const double *wl, const double *wr, double glc, double gle,
                                        double grc, double gre, const GasConsts &gc,
                                        double *flx) {
  if (RS == RS_HLLE) {
    solve_hlle<CONSTG>(wl, wr, glc, gle, grc, gre, gc, flx);
  } else if (RS == RS_HLLC) {
#if APH_EXACT
    solve_hllc_exact<false, TAME>(wl, wr, glc, gle, grc, gre, flx);
#else
    solve_hllc<CONSTG, false>(wl, wr, glc, gle, grc, gre, gc, flx);
#endif
  } else if (RS == RS_LHLLC) {
#if APH_EXACT
    solve_hllc_exact<true, TAME>(wl, wr, glc, gle, grc, gre, flx);
#else
    solve_hllc<CONSTG, true>(wl, wr, glc, gle, grc, gre, gc, flx);
#endif
  } else {
#pragma unroll
    for (int n = 0; n < NHYDRO; ++n) flx[n] = 0.0;
  }
}

// EstimateTimestep per-cell candidate (hydro.cpp:384-415): min over active directions
// of dx_d / (|v_d| + lambda).  dt_cell below is the form the stage kernel uses.
__device__ __forceinline__ double dt_candidate(const double *w, double e_cons, const double *dx,
                                               int ndim, double gm1) {
  const double e_internal =
      (e_cons - 0.5 * w[IDN] * (w[IV1] * w[IV1] + w[IV2] * w[IV2] + w[IV3] * w[IV3])) / w[IDN];
  const double bulkmod = eos_bulk_modulus(gm1, w[IDN], e_internal);
  double gamma_c, rat;  // bulkmod / p, (e_internal + c^2) rho / p
  div2(bulkmod, (e_internal + C_LIGHT2) * w[IDN], w[IPR], gamma_c, rat);
  const double lam = C_LIGHT * sqrt(gamma_c / (1 + rat));
  double m = dx[0] / (dabs(w[IV1]) + lam);
  if (ndim > 1) {
    const double c2 = dx[1] / (dabs(w[IV2]) + lam);
    m = lt(c2, m) ? c2 : m;
  }
  if (ndim > 2) {
    const double c3 = dx[2] / (dabs(w[IV3]) + lam);
    m = lt(c3, m) ? c3 : m;
  }
  return m;
}

// dt candidate of a cell just converted by cons_to_prim_cell (floored: its return value).
// Fast mode with the floors inactive: lambda is the c-limited sound speed of the constant
// gamma (the same quantity: rho e = p / gm1), and one reciprocal of the largest rate
// (|v_d| + lambda) / dx_d replaces a division per direction.
__device__ __forceinline__ double dt_cell(const double *w, double e_cons, const double *dx, int ndim,
                                          const GasConsts &gc, bool floored) {
#if APH_EXACT
  return dt_candidate(w, e_cons, dx, ndim, gc.gm1);
#else
  if (floored) return dt_candidate(w, e_cons, dx, ndim, gc.gm1);
  const double lam = sound_speed<true>(w[IDN], w[IPR], 0.0, 0.0, gc);
  double r = (dabs(w[IV1]) + lam) / dx[0];
  if (ndim > 1) {
    const double r2 = (dabs(w[IV2]) + lam) / dx[1];
    r = lt(r, r2) ? r2 : r;
  }
  if (ndim > 2) {
    const double r3 = (dabs(w[IV3]) + lam) / dx[2];
    r = lt(r, r3) ? r3 : r;
  }
  return 1.0 / r;
#endif
}

}  // namespace aph
