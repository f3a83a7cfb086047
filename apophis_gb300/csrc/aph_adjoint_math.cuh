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
  // left flux
  for (int n = 0; n < 5; ++n) gwl[n] = 0.0, gwr[n] = 0.0;
  double gvxl = 0.0, gvxr = 0.0, gel = 0.0, ger = 0.0;
  gwl[IDN] += gfl[0] * vxl; gvxl += gfl[0] * wl[IDN];
  gwl[IDN] += gfl[1] * wl[IV1] * vxl; gwl[IV1] += gfl[1] * wl[IDN] * vxl;
  gvxl += gfl[1] * wl[IDN] * wl[IV1]; gwl[IPR] += gfl[1];
  gwl[IDN] += gfl[2] * wl[IV2] * vxl; gwl[IV2] += gfl[2] * wl[IDN] * vxl; gvxl += gfl[2] * wl[IDN] * wl[IV2];
  gwl[IDN] += gfl[3] * wl[IV3] * vxl; gwl[IV3] += gfl[3] * wl[IDN] * vxl; gvxl += gfl[3] * wl[IDN] * wl[IV3];
  gel += gfl[4] * vxl; gvxl += gfl[4] * el; gwl[IPR] += gfl[4] * wl[IV1]; gwl[IV1] += gfl[4] * wl[IPR];
  // right flux
  gwr[IDN] += gfr[0] * vxr; gvxr += gfr[0] * wr[IDN];
  gwr[IDN] += gfr[1] * wr[IV1] * vxr; gwr[IV1] += gfr[1] * wr[IDN] * vxr;
  gvxr += gfr[1] * wr[IDN] * wr[IV1]; gwr[IPR] += gfr[1];
  gwr[IDN] += gfr[2] * wr[IV2] * vxr; gwr[IV2] += gfr[2] * wr[IDN] * vxr; gvxr += gfr[2] * wr[IDN] * wr[IV2];
  gwr[IDN] += gfr[3] * wr[IV3] * vxr; gwr[IV3] += gfr[3] * wr[IDN] * vxr; gvxr += gfr[3] * wr[IDN] * wr[IV3];
  ger += gfr[4] * vxr; gvxr += gfr[4] * er; gwr[IPR] += gfr[4] * wr[IV1]; gwr[IV1] += gfr[4] * wr[IPR];
  // vxl = ul - bm, vxr = ur - bp
  gwl[IV1] += gvxl; gbm -= gvxl;
  gwr[IV1] += gvxr; gbp -= gvxr;
  // energies
  gwl[IPR] += gel * igm1; gwl[IDN] += gel * 0.5 * kel;
  gwl[IV1] += gel * wl[IDN] * wl[IV1]; gwl[IV2] += gel * wl[IDN] * wl[IV2]; gwl[IV3] += gel * wl[IDN] * wl[IV3];
  gwr[IPR] += ger * igm1; gwr[IDN] += ger * 0.5 * ker;
  gwr[IV1] += ger * wr[IDN] * wr[IV1]; gwr[IV2] += ger * wr[IDN] * wr[IV2]; gwr[IV3] += ger * wr[IDN] * wr[IV3];
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

// ---- HLLC (hydro_hllc.hpp:161-282) -----------------------------------------------------------
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
  const double wxl = ul - bm, wxr = ur - bp;
  double fl[5], fr[5];
  fl[0] = rl * wxl;
  fr[0] = rr * wxr;
  fl[1] = rl * ul * wxl + pl;
  fr[1] = rr * ur * wxr + pr;
  fl[2] = rl * vl * wxl;
  fr[2] = rr * vr * wxr;
  fl[3] = rl * zl * wxl;
  fr[3] = rr * zr * wxr;
  fl[4] = el * wxl + pl * ul;
  fr[4] = er * wxr + pr * ur;
  const bool sp = !is_neg(sstar);
  double cl_, cr_, ustar, idn;
  if (sp) {
    idn = 1.0 / (sstar - bm);
    cl_ = sstar * idn;
    cr_ = 0.0;
    ustar = -bm * idn;
  } else {
    idn = 1.0 / (bp - sstar);
    cl_ = 0.0;
    cr_ = -sstar * idn;
    ustar = bp * idn;
  }
  // reverse: flx = cl_ fl + cr_ fr + (0, ustar cp, 0, 0, ustar cp sstar)
  double gfl[5], gfr[5];
  double gcl_ = 0.0, gcr_ = 0.0;
#pragma unroll
  for (int n = 0; n < 5; ++n) {
    gfl[n] = gf[n] * cl_;
    gfr[n] = gf[n] * cr_;
    gcl_ += gf[n] * fl[n];
    gcr_ += gf[n] * fr[n];
  }
  double gustar = gf[1] * cp + gf[4] * cp * sstar;
  double gcp = gf[1] * ustar + gf[4] * ustar * sstar;
  double gsstar = gf[4] * ustar * cp;
  double gbp = 0.0, gbm = 0.0;
  if (sp) {
    // cl_ = s/(s - bm), ustar = -bm/(s - bm)
    const double i2 = idn * idn;
    gsstar += gcl_ * (-bm) * i2 + gustar * bm * i2;
    gbm += gcl_ * sstar * i2 + gustar * (-sstar) * i2;
  } else {
    // cr_ = -s/(bp - s), ustar = bp/(bp - s)
    const double i2 = idn * idn;
    gsstar += gcr_ * (-bp) * i2 + gustar * bp * i2;
    gbp += gcr_ * sstar * i2 + gustar * (-sstar) * i2;
  }
  for (int n = 0; n < 5; ++n) gwl[n] = 0.0, gwr[n] = 0.0;
  double gwxl = 0.0, gwxr = 0.0, gel = 0.0, ger = 0.0;
  gwl[IDN] += gfl[0] * wxl; gwxl += gfl[0] * rl;
  gwl[IDN] += gfl[1] * ul * wxl; gwl[IV1] += gfl[1] * rl * wxl; gwxl += gfl[1] * rl * ul; gwl[IPR] += gfl[1];
  gwl[IDN] += gfl[2] * vl * wxl; gwl[IV2] += gfl[2] * rl * wxl; gwxl += gfl[2] * rl * vl;
  gwl[IDN] += gfl[3] * zl * wxl; gwl[IV3] += gfl[3] * rl * wxl; gwxl += gfl[3] * rl * zl;
  gel += gfl[4] * wxl; gwxl += gfl[4] * el; gwl[IPR] += gfl[4] * ul; gwl[IV1] += gfl[4] * pl;
  gwr[IDN] += gfr[0] * wxr; gwxr += gfr[0] * rr;
  gwr[IDN] += gfr[1] * ur * wxr; gwr[IV1] += gfr[1] * rr * wxr; gwxr += gfr[1] * rr * ur; gwr[IPR] += gfr[1];
  gwr[IDN] += gfr[2] * vr * wxr; gwr[IV2] += gfr[2] * rr * wxr; gwxr += gfr[2] * rr * vr;
  gwr[IDN] += gfr[3] * zr * wxr; gwr[IV3] += gfr[3] * rr * wxr; gwxr += gfr[3] * rr * zr;
  ger += gfr[4] * wxr; gwxr += gfr[4] * er; gwr[IPR] += gfr[4] * ur; gwr[IV1] += gfr[4] * pr;
  // wxl = ul - bm, wxr = ur - bp
  gwl[IV1] += gwxl; gbm -= gwxl;
  gwr[IV1] += gwxr; gbp -= gwxr;
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
  // energies
  gwl[IPR] += gel * igm1; gwl[IDN] += gel * 0.5 * kel;
  gwl[IV1] += gel * rl * ul; gwl[IV2] += gel * rl * vl; gwl[IV3] += gel * rl * zl;
  gwr[IPR] += ger * igm1; gwr[IDN] += ger * 0.5 * ker;
  gwr[IV1] += ger * rr * ur; gwr[IV2] += ger * rr * vr; gwr[IV3] += ger * rr * zr;
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
