// aph_adjoint_math.cuh -- hand-written reverse-mode derivatives of the hydro step's
// pointwise pieces: ConsToPrim (ideal gas, floors inactive), PLM, donor cell, and the
// HLLE / HLLC fluxes with their wave-speed and contact branches.
//
// Each *_vjp routine recomputes its forward intermediates and propagates the adjoint of
// its outputs to its inputs (vector-Jacobian product).  The branches taken are the
// forward's branches: at a kink (limiter switch, wave-speed clamp, contact direction)
// the derivative of the active branch is used.  The fluxes are differentiated through the
// fast-mode forward formulas (constant adiabatic index of the pack, sound speed
// sqrt(C^2 gamma p / (p (1 + 1/gm1) + rho C^2))), the same quantity as the reference's
// c-limited sound speed.
#pragma once
#include "aph_math.cuh"

namespace aph {

// ---- ConsToPrim: W = (rho, m/rho, p = gm1 (E - |m|^2 / (2 rho))) -----------------------
// The Jacobian depends on rho and v only, so it is evaluated from the primitives w.
__device__ __forceinline__ void cons_to_prim_vjp(const double *w, const double *gw, double gm1,
                                                 double *gu) {
  const double di = 1.0 / w[IDN];
  const double v1 = w[IV1], v2 = w[IV2], v3 = w[IV3];
  const double gp = gw[IPR];
  const double v2sum = v1 * v1 + v2 * v2 + v3 * v3;
  gu[IDN] = gw[IDN] - (gw[IV1] * v1 + gw[IV2] * v2 + gw[IV3] * v3) * di + gp * 0.5 * gm1 * v2sum;
  gu[IM1] = gw[IV1] * di - gp * gm1 * v1;
  gu[IM2] = gw[IV2] * di - gp * gm1 * v2;
  gu[IM3] = gw[IV3] * di - gp * gm1 * v3;
  gu[IEN] = gp * gm1;
}

// ---- PLM (plm_simple.hpp:15-32) ---------------------------------------------------------
// Forward with the reciprocal kept: dqm = dq2 r, r = 1/(dql + dqr) where the slopes agree in
// sign, r = 0 where the limiter returns 0.
__device__ __forceinline__ double plm_keep(double q_im1, double q_i, double q_ip1, double &ql,
                                           double &qr) {
  const double dql = q_i - q_im1, dqr = q_ip1 - q_i;
  const double dq2 = dql * dqr;
  double r = 0.0, dqm = 0.0;
  if (is_pos(dq2)) {
    r = 1.0 / (dql + dqr);
    dqm = dq2 * r;
  }
  ql = q_i + dqm;
  qr = q_i - dqm;
  return r;
}

// gL is the adjoint of ql_{i+1}, gR of qr_i; r as plm_keep returned it.
__device__ __forceinline__ void plm_vjp(double q_im1, double q_i, double q_ip1, double r, double gL,
                                        double gR, double &g_im1, double &g_i, double &g_ip1) {
  g_i = gL + gR;
  g_im1 = 0.0;
  g_ip1 = 0.0;
  if (r != 0.0) {
    const double dql = q_i - q_im1, dqr = q_ip1 - q_i;
    const double gr2 = (gL - gR) * r * r;  // adjoint of dqm times 1/(dql + dqr)^2
    const double gdql = gr2 * dqr * dqr;   // d dqm / d dql = dqr^2 / s^2
    const double gdqr = gr2 * dql * dql;   // d dqm / d dqr = dql^2 / s^2
    g_i += gdql - gdqr;
    g_im1 = -gdql;
    g_ip1 = gdqr;
  }
}

// ---- PPM (ppm_simple.hpp:32-161, in the face/cell split of aph_math.cuh) --------------------
// The forward is piecewise linear in q except the extremum limiter's ratio rho = qe / d2qf,
// so the reverse records the branch each face and cell took and applies the transposed
// linear map of that branch (and the quotient rule for rho).
constexpr int PF_OPEN = 0, PF_AVG = 1, PF_D2M = 2, PF_D20 = 3, PF_QA = 4;

// ppm_face (fast arithmetic) returning the branch: OPEN (unlimited), or limited with
// qd = 0 (AVG), C2 d2(f-1) (D2M), C2 d2(f) (D20), or qa (QA).
__device__ __forceinline__ double ppm_face_code(double qm1, double q0, double ddm1, double dd0,
                                                double d2m1, double d20, int &code) {
  const double avg = 0.5 * (qm1 + q0);
  double dph = fma(ddm1 - dd0, 1.0 / 6.0, avg);
  const double qa = 3.0 * (qm1 + q0 - 2.0 * dph);
  code = PF_OPEN;
  if (strictly_outside(dph, qm1, q0)) {  // the forward's test (ppm_face, fast mode)
    double qd = 0.0;
    code = PF_AVG;
    const bool sa = is_neg(qa);
    if (sa == is_neg(d2m1) && sa == is_neg(d20)) {
      const unsigned long long mb = mag(d2m1), mc = mag(d20);
      const bool pick_c = mc < mb;
      const unsigned long long mm = mag(PPM_C2 * from_bits(pick_c ? mc : mb)), ma = mag(qa);
      if (ma < mm) {
        qd = qa;
        code = PF_QA;
      } else {
        qd = flip_if(from_bits(mm), sa);
        code = pick_c ? PF_D20 : PF_D2M;
      }
    }
    dph = fma(qd, -1.0 / 6.0, avg);
  }
  return dph;
}

// d dph / d (q[f-2], q[f-1], q[f], q[f+1]) of a face with the given branch (dd and d2 are
// linear; the QA branch gives back the unlimited value).
__device__ __forceinline__ void ppm_face_coef(int code, double c[4]) {
  constexpr double a = 1.0 / 12.0, b = PPM_C2 / 6.0;
  if (code == PF_AVG) {
    c[0] = 0.0; c[1] = 0.5; c[2] = 0.5; c[3] = 0.0;
  } else if (code == PF_D2M) {
    c[0] = -b; c[1] = 0.5 + 2.0 * b; c[2] = 0.5 - b; c[3] = 0.0;
  } else if (code == PF_D20) {
    c[0] = 0.0; c[1] = 0.5 - b; c[2] = 0.5 + 2.0 * b; c[3] = -b;
  } else {
    c[0] = -a; c[1] = 7.0 * a; c[2] = 7.0 * a; c[3] = -a;
  }
}

// ppm_cell (fast arithmetic) returning its branch: bit 0 extremum; extremum: bits 1-3 the
// source of qe (0 none, 1..3 C2 d2 of cell i-1, i, i+1, 4 d2qf), bit 4 the ratio applied;
// monotone: bit 1 qr steepened, bit 2 ql steepened.  rho: the ratio used.
__device__ __forceinline__ void ppm_cell_code(double q_im2, double q_im1, double q_i, double q_ip1,
                                              double q_ip2, double d2m1, double d20, double d2p1,
                                              double dph_lo, double dph_hi, double &ql, double &qr,
                                              int &code, double &rho) {
  const double d2qf = 6.0 * (dph_lo + dph_hi - 2.0 * q_i);
  qr = dph_lo;
  ql = dph_hi;
  const double dqf_minus = q_i - qr;
  const double dqf_plus = ql - q_i;
  code = 0;
  rho = 0.0;
  if (!strictly_between(qr, q_i, ql) || !strictly_between(q_im1, q_i, q_ip1)) {  // as ppm_cell
    code = 1;
    double qe = 0.0;
    int src = 0;
    const bool sd = is_neg(d2qf);
    if (sd == is_neg(d2m1) && sd == is_neg(d20) && sd == is_neg(d2p1)) {
      unsigned long long m = mag(d2m1);
      int k = 1;
      const unsigned long long m0 = mag(d20), m1 = mag(d2p1);
      if (m0 < m) { m = m0; k = 2; }
      if (m1 < m) { m = m1; k = 3; }
      const unsigned long long ms = mag(PPM_C2 * from_bits(m)), md = mag(d2qf);
      if (md < ms) {
        qe = d2qf;
        src = 4;
      } else {
        qe = flip_if(from_bits(ms), sd);
        src = k;
      }
    }
    unsigned long long mx = mag(q_im2);
    const unsigned long long a1 = mag(q_im1), a2 = mag(q_i), a3 = mag(q_ip1), a4 = mag(q_ip2);
    mx = a1 > mx ? a1 : mx;
    mx = a2 > mx ? a2 : mx;
    mx = a3 > mx ? a3 : mx;
    mx = a4 > mx ? a4 : mx;
    if (mag(d2qf) > mag(1.0e-12 * from_bits(mx))) rho = qe / d2qf;
    code |= src << 1;
    if (le(rho, 1.0 - 1.0e-12)) {
      qr = fma(-rho, dqf_minus, q_i);
      ql = fma(rho, dqf_plus, q_i);
      code |= 16;
    }
  } else {
    if (mag(dqf_minus) >= twice_mag(dqf_plus)) {
      qr = q_i - 2.0 * dqf_plus;
      code |= 2;
    }
    if (mag(dqf_plus) >= twice_mag(dqf_minus)) {
      ql = q_i + 2.0 * dqf_minus;
      code |= 4;
    }
  }
}

// Reverse of ppm_cell_code: gL, gR adjoints of ql_{i+1}, qr_i; out: gq (q_{i-2..i+2}) and the
// adjoints of the two face values.
__device__ __forceinline__ void ppm_cell_vjp(double q_i, double dph_lo, double dph_hi, int code,
                                             double rho, double gL, double gR, double gq[5],
                                             double &g_lo, double &g_hi) {
#pragma unroll
  for (int k = 0; k < 5; ++k) gq[k] = 0.0;
  g_lo = 0.0;
  g_hi = 0.0;
  if (code & 1) {
    if (code & 16) {  // ql = q_i + rho (dph_hi - q_i), qr = q_i - rho (q_i - dph_lo)
      gq[2] += (gL + gR) * (1.0 - rho);
      g_hi += gL * rho;
      g_lo += gR * rho;
      const int src = (code >> 1) & 7;
      if (rho != 0.0 && src >= 1 && src <= 3) {  // rho = C2 d2(i + src - 2) / d2qf
        const double d2qf = 6.0 * (dph_lo + dph_hi - 2.0 * q_i);
        const double g_rho = gL * (dph_hi - q_i) - gR * (q_i - dph_lo);
        const double g_qe = g_rho / d2qf;
        const double g_d2qf = -g_qe * rho;
        g_lo += 6.0 * g_d2qf;
        g_hi += 6.0 * g_d2qf;
        gq[2] -= 12.0 * g_d2qf;
        // d2 of cell i + src - 2 is q[c-1] + q[c+1] - 2 q[c], c at gq index src
        const double gd = PPM_C2 * g_qe;
        if (src == 1) {
          gq[0] += gd; gq[2] += gd; gq[1] -= 2.0 * gd;
        } else if (src == 2) {
          gq[1] += gd; gq[3] += gd; gq[2] -= 2.0 * gd;
        } else {
          gq[2] += gd; gq[4] += gd; gq[3] -= 2.0 * gd;
        }
      }
    } else {
      g_hi += gL;
      g_lo += gR;
    }
  } else {
    if (code & 2) {  // qr = 3 q_i - 2 dph_hi
      gq[2] += 3.0 * gR;
      g_hi -= 2.0 * gR;
    } else {
      g_lo += gR;
    }
    if (code & 4) {  // ql = 3 q_i - 2 dph_lo
      gq[2] += 3.0 * gL;
      g_lo -= 2.0 * gL;
    } else {
      g_hi += gL;
    }
  }
}

// ---- sound speed c = sqrt(N/D), N = C^2 gamma p, D = p (1 + 1/gm1) + rho C^2 ------------
// ip = 1/p; 1/D = c^2 / N = c^2 ip / (C^2 gamma), so no division beyond ip.
struct SoundSpeed {
  double c, dc_dp, dc_drho;
};
__device__ __forceinline__ SoundSpeed sound_speed_d(double rho, double p, double ip,
                                                    const GasConsts &gc, double ic2g) {
  const double N = gc.c2g * p;
  const double D = fma(p, gc.one_igm1, rho * C_LIGHT2);
  const double c = N * rsqrt(N * D);
  const double iD = c * c * ip * ic2g;
  SoundSpeed s;
  s.c = c;
  s.dc_dp = 0.5 * c * (ip - gc.one_igm1 * iD);
  s.dc_drho = -0.5 * c * C_LIGHT2 * iD;
  return s;
}

// Adjoint of one side's physical flux  F = (rho vx, rho u vx + p, rho v vx, rho z vx, e vx + p u)
// with vx = u - b and e = p/gm1 + rho |v|^2 / 2, for the flux adjoint g: adds to gw
// (rho, u, v, z, p) and returns the adjoint of vx (the b-dependence is the caller's).
__device__ __forceinline__ double side_flux_vjp(const double *w, double vx, double e, double igm1,
                                                const double *g, double *gw) {
  const double rho = w[IDN], u = w[IV1], v = w[IV2], z = w[IV3], p = w[IPR];
  const double A = g[0] + g[1] * u + g[2] * v + g[3] * z;  // shared by d/drho and d/dvx
  const double rvx = rho * vx;
  const double ge = g[4] * vx;                               // adjoint of e
  const double rge = rho * ge;
  gw[IDN] += A * vx + ge * 0.5 * (u * u + v * v + z * z);
  gw[IV1] += g[1] * rvx + g[4] * p + rge * u;
  gw[IV2] += g[2] * rvx + rge * v;
  gw[IV3] += g[3] * rvx + rge * z;
  gw[IPR] += g[1] + g[4] * u + ge * igm1;
  return rho * A + g[4] * e;
}

// ---- HLLE (hydro_hlle.hpp:28-133) ----------------------------------------------------------
// w*: (rho, v_n, v_t1, v_t2, p); gf: adjoint of the 5 flux components; gwl/gwr: output.
__device__ void hlle_vjp(const double *wl, const double *wr, const GasConsts &gc, double ic2g,
                         const double *gf, double *gwl, double *gwr) {
  const double igm1 = gc.igm1;
  const double ipl = 1.0 / wl[IPR], ipr = 1.0 / wr[IPR];
  const SoundSpeed sl = sound_speed_d(wl[IDN], wl[IPR], ipl, gc, ic2g);
  const SoundSpeed sr = sound_speed_d(wr[IDN], wr[IPR], ipr, gc, ic2g);
  const double cl = sl.c, cr = sr.c;
  const double kel = wl[IV1] * wl[IV1] + wl[IV2] * wl[IV2] + wl[IV3] * wl[IV3];
  const double ker = wr[IV1] * wr[IV1] + wr[IV2] * wr[IV2] + wr[IV3] * wr[IV3];
  const double el = wl[IPR] * igm1 + 0.5 * wl[IDN] * kel;
  const double er = wr[IPR] * igm1 + 0.5 * wr[IDN] * ker;
  const double rhoa = .5 * (wl[IDN] + wr[IDN]);
  const double ca = .5 * (cl + cr);
  const double pmid = .5 * (wl[IPR] + wr[IPR] + (wl[IV1] - wr[IV1]) * rhoa * ca);
  const bool bl = gt(pmid, wl[IPR]), br = gt(pmid, wr[IPR]);
  const double k = gc.hlle_k;
  const double ql = bl ? 1.0 + k * (pmid * ipl - 1.0) : 1.0;
  const double qr = br ? 1.0 + k * (pmid * ipr - 1.0) : 1.0;
  const double al = wl[IV1] - cl * ql;
  const double ar = wr[IV1] + cr * qr;
  const bool bpos = is_pos(ar), bneg = is_neg(al);
  const double bp = bpos ? ar : 0.0;
  const double bm = bneg ? al : 0.0;
  const double vxl = wl[IV1] - bm, vxr = wr[IV1] - bp;
  double fl[5], fr[5];
  fl[0] = wl[IDN] * vxl;
  fr[0] = wr[IDN] * vxr;
  fl[1] = wl[IDN] * wl[IV1] * vxl + wl[IPR];
  fr[1] = wr[IDN] * wr[IV1] * vxr + wr[IPR];
  fl[2] = wl[IDN] * wl[IV2] * vxl;
  fr[2] = wr[IDN] * wr[IV2] * vxr;
  fl[3] = wl[IDN] * wl[IV3] * vxl;
  fr[3] = wr[IDN] * wr[IV3] * vxr;
  fl[4] = el * vxl + wl[IPR] * wl[IV1];
  fr[4] = er * vxr + wr[IPR] * wr[IV1];
  const bool has = (mag(bp) | mag(bm)) != 0ULL;
  const double ibpm = has ? 1.0 / (bp - bm) : 0.0;
  const double tmp = has ? 0.5 * (bp + bm) * ibpm : 0.0;
  // reverse
  double gfl[5], gfr[5], gtmp = 0.0;
#pragma unroll
  for (int n = 0; n < 5; ++n) {
    gfl[n] = gf[n] * (0.5 + tmp);
    gfr[n] = gf[n] * (0.5 - tmp);
    gtmp += gf[n] * (fl[n] - fr[n]);
  }
  double gbp = 0.0, gbm = 0.0;
  if (has) {
    gbp = gtmp * (-bm) * ibpm * ibpm;
    gbm = gtmp * bp * ibpm * ibpm;
  }
  for (int n = 0; n < 5; ++n) gwl[n] = 0.0, gwr[n] = 0.0;
  // fluxes of both sides (vxl = ul - bm, vxr = ur - bp)
  const double gvxl = side_flux_vjp(wl, vxl, el, igm1, gfl, gwl);
  const double gvxr = side_flux_vjp(wr, vxr, er, igm1, gfr, gwr);
  gwl[IV1] += gvxl; gbm -= gvxl;
  gwr[IV1] += gvxr; gbp -= gvxr;
  // clamps
  const double gar = bpos ? gbp : 0.0;
  const double gal = bneg ? gbm : 0.0;
  // al = ul - cl ql ; ar = ur + cr qr
  gwl[IV1] += gal;
  double gcl = -gal * ql, gql = -gal * cl;
  gwr[IV1] += gar;
  double gcr = gar * qr, gqr = gar * cr;
  // ql, qr
  double gpmid = 0.0;
  if (bl) {
    gpmid += gql * k * ipl;
    gwl[IPR] -= gql * k * pmid * ipl * ipl;
  }
  if (br) {
    gpmid += gqr * k * ipr;
    gwr[IPR] -= gqr * k * pmid * ipr * ipr;
  }
  // pmid = 0.5 (pl + pr + (ul - ur) rhoa ca)
  gwl[IPR] += 0.5 * gpmid;
  gwr[IPR] += 0.5 * gpmid;
  const double du = wl[IV1] - wr[IV1];
  gwl[IV1] += 0.5 * gpmid * rhoa * ca;
  gwr[IV1] -= 0.5 * gpmid * rhoa * ca;
  const double grhoa = 0.5 * gpmid * du * ca;
  const double gca = 0.5 * gpmid * du * rhoa;
  gwl[IDN] += 0.5 * grhoa;
  gwr[IDN] += 0.5 * grhoa;
  gcl += 0.5 * gca;
  gcr += 0.5 * gca;
  gwl[IPR] += gcl * sl.dc_dp; gwl[IDN] += gcl * sl.dc_drho;
  gwr[IPR] += gcr * sr.dc_dp; gwr[IDN] += gcr * sr.dc_drho;
}

// ---- HLLC (hydro_hllc.hpp:14-146) -----------------------------------------------------------
__device__ void hllc_vjp(const double *wl, const double *wr, const GasConsts &gc, double ic2g,
                         const double *gf, double *gwl, double *gwr) {
  const double igm1 = gc.igm1;
  const double ipl = 1.0 / wl[IPR], ipr = 1.0 / wr[IPR];
  const SoundSpeed sdl = sound_speed_d(wl[IDN], wl[IPR], ipl, gc, ic2g);
  const SoundSpeed sdr = sound_speed_d(wr[IDN], wr[IPR], ipr, gc, ic2g);
  const double cl = sdl.c, cr = sdr.c;
  const double rl = wl[IDN], ul = wl[IV1], vl = wl[IV2], zl = wl[IV3], pl = wl[IPR];
  const double rr = wr[IDN], ur = wr[IV1], vr = wr[IV2], zr = wr[IV3], pr = wr[IPR];
  const double kel = ul * ul + vl * vl + zl * zl, ker = ur * ur + vr * vr + zr * zr;
  const double el = pl * igm1 + 0.5 * rl * kel;
  const double er = pr * igm1 + 0.5 * rr * ker;
  const double rhoa = .5 * (rl + rr);
  const double ca = .5 * (cl + cr);
  const double pstar = .5 * (pl + pr) - .5 * (ur - ul) * rhoa * ca;
  const double k = gc.hllc_k;
  const bool bl = gt(pstar, pl), br = gt(pstar, pr);
  const double argl = bl ? 1.0 + k * (pstar * ipl - 1.0) : 1.0;
  const double argr = br ? 1.0 + k * (pstar * ipr - 1.0) : 1.0;
  const double iql = bl ? rsqrt(argl) : 1.0;  // q = arg / sqrt(arg), 1/q kept for the reverse
  const double iqr = br ? rsqrt(argr) : 1.0;
  const double ql = bl ? argl * iql : 1.0;
  const double qr = br ? argr * iqr : 1.0;
  const double sl = ul - cl * ql;
  const double sr = ur + cr * qr;
  const bool bpos = is_pos(sr), bneg = is_neg(sl);
  const double bp = bpos ? sr : TINY_NUMBER;
  const double bm = bneg ? sl : -TINY_NUMBER;
  const double vxl = ul - sl, vxr = ur - sr;
  const double tl = pl + vxl * rl * ul;
  const double tr = pr + vxr * rr * ur;
  const double ml = rl * vxl;
  const double mr = -(rr * vxr);
  const double imm = 1.0 / (ml + mr);
  const double sstar = (tl - tr) * imm;
  const double cp0 = (ml * tr + mr * tl) * imm;
  const bool cpos = is_pos(cp0);
  const double cp = cpos ? cp0 : 0.0;
  // flx = c_s F_s(w_s) + (0, ustar cp, 0, 0, ustar cp sstar) with the upwind side s of the
  // contact (left with b = bm when sstar >= 0, else right with b = bp); the other side's
  // weight is exactly 0, so only side s is differentiated
  const bool sp = !is_neg(sstar);
  double ws[5];
#pragma unroll
  for (int n = 0; n < 5; ++n) ws[n] = sp ? wl[n] : wr[n];
  const double b = sp ? bm : bp;
  const double es = sp ? el : er;
  const double wx = ws[IV1] - b;
  double fs[5];
  fs[0] = ws[IDN] * wx;
  fs[1] = ws[IDN] * ws[IV1] * wx + ws[IPR];
  fs[2] = ws[IDN] * ws[IV2] * wx;
  fs[3] = ws[IDN] * ws[IV3] * wx;
  fs[4] = es * wx + ws[IPR] * ws[IV1];
  // c = sstar / (sstar - b), ustar = -b / (sstar - b)
  const double idn = 1.0 / (sstar - b);
  const double cs = sstar * idn;
  const double ustar = -b * idn;
  double gfs[5], gcs = 0.0;
#pragma unroll
  for (int n = 0; n < 5; ++n) {
    gfs[n] = gf[n] * cs;
    gcs += gf[n] * fs[n];
  }
  double gustar = gf[1] * cp + gf[4] * cp * sstar;
  double gcp = gf[1] * ustar + gf[4] * ustar * sstar;
  double gsstar = gf[4] * ustar * cp;
  // d c / d sstar = -b idn^2, d c / d b = sstar idn^2; d ustar / d sstar = b idn^2,
  // d ustar / d b = -sstar idn^2
  const double i2 = idn * idn;
  gsstar += (gustar - gcs) * b * i2;
  const double gb_w = (gcs - gustar) * sstar * i2;
  double gws[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  const double gwx = side_flux_vjp(ws, wx, es, igm1, gfs, gws);
  gws[IV1] += gwx;
  const double gb = gb_w - gwx;
  for (int n = 0; n < 5; ++n) {
    gwl[n] = sp ? gws[n] : 0.0;
    gwr[n] = sp ? 0.0 : gws[n];
  }
  double gbm = sp ? gb : 0.0, gbp = sp ? 0.0 : gb;
  // cp = max(cp0, 0)
  const double gcp0 = cpos ? gcp : 0.0;
  // sstar = (tl - tr) imm; cp0 = (ml tr + mr tl) imm; imm = 1/(ml + mr)
  double gtl = gsstar * imm + gcp0 * mr * imm;
  double gtr = -gsstar * imm + gcp0 * ml * imm;
  const double gimm = gsstar * (tl - tr) + gcp0 * (ml * tr + mr * tl);
  const double gsum = -gimm * imm * imm;
  double gml = gcp0 * tr * imm + gsum;
  double gmr = gcp0 * tl * imm + gsum;
  // ml = rl vxl ; mr = -(rr vxr)
  double gvxl = gml * rl, gvxr = -gmr * rr;
  gwl[IDN] += gml * vxl;
  gwr[IDN] -= gmr * vxr;
  // tl = pl + vxl rl ul ; tr = pr + vxr rr ur
  gwl[IPR] += gtl; gvxl += gtl * rl * ul; gwl[IDN] += gtl * vxl * ul; gwl[IV1] += gtl * vxl * rl;
  gwr[IPR] += gtr; gvxr += gtr * rr * ur; gwr[IDN] += gtr * vxr * ur; gwr[IV1] += gtr * vxr * rr;
  // vxl = ul - sl ; vxr = ur - sr
  gwl[IV1] += gvxl;
  double gsl = -gvxl;
  gwr[IV1] += gvxr;
  double gsr = -gvxr;
  // bp = sr or TINY ; bm = sl or -TINY
  if (bpos) gsr += gbp;
  if (bneg) gsl += gbm;
  // sl = ul - cl ql ; sr = ur + cr qr
  gwl[IV1] += gsl;
  double gcl = -gsl * ql, gql = -gsl * cl;
  gwr[IV1] += gsr;
  double gcr = gsr * qr, gqr = gsr * cr;
  // ql = sqrt(1 + k (pstar/pl - 1)) when pstar > pl
  double gpstar = 0.0;
  if (bl) {
    const double garg = gql * 0.5 * iql;
    gpstar += garg * k * ipl;
    gwl[IPR] -= garg * k * pstar * ipl * ipl;
  }
  if (br) {
    const double garg = gqr * 0.5 * iqr;
    gpstar += garg * k * ipr;
    gwr[IPR] -= garg * k * pstar * ipr * ipr;
  }
  // pstar = 0.5 (pl + pr) - 0.5 (ur - ul) rhoa ca
  gwl[IPR] += 0.5 * gpstar;
  gwr[IPR] += 0.5 * gpstar;
  gwr[IV1] -= 0.5 * gpstar * rhoa * ca;
  gwl[IV1] += 0.5 * gpstar * rhoa * ca;
  const double dd = ur - ul;
  const double grhoa = -0.5 * gpstar * dd * ca;
  const double gca = -0.5 * gpstar * dd * rhoa;
  gwl[IDN] += 0.5 * grhoa;
  gwr[IDN] += 0.5 * grhoa;
  gcl += 0.5 * gca;
  gcr += 0.5 * gca;
  gwl[IPR] += gcl * sdl.dc_dp; gwl[IDN] += gcl * sdl.dc_drho;
  gwr[IPR] += gcr * sdr.dc_dp; gwr[IDN] += gcr * sdr.dc_drho;
}

}  // namespace aph
