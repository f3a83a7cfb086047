// ref_pin.cpp -- the reference's own reconstruction and Riemann-solver code, compiled from
// its sources, behind a small C interface.
//
// TEST INFRASTRUCTURE ONLY.  oracle/build_ref.py compiles this file together with the
// reference's headers (src/recon/{dc,plm,ppm}_simple.hpp, src/hydro/rsolvers/hydro_{none,
// hlle,hllc,lhllc}.hpp, src/main.hpp, all read where they lie in the reference checkout) and
// the stand-ins of oracle/ref_shim/ into oracle/_ref/libref_pin.so, with the oracle's flags
// (-O2 -ffp-contract=off).  tests/test_ref_pin.py then requires the oracle's restatement to
// equal this code bit for bit.  Nothing in the product links or calls it.
#include <vector>

#include "recon/dc_simple.hpp"
#include "recon/plm_simple.hpp"
#include "recon/ppm_simple.hpp"
#include "hydro/rsolvers/hydro_hlle.hpp"
#include "hydro/rsolvers/hydro_hllc.hpp"
#include "hydro/rsolvers/hydro_lhllc.hpp"
#include "hydro/rsolvers/hydro_none.hpp"

namespace {

using parthenon::ScratchPad2D;
using parthenon::VariableFluxPack;
using parthenon::VariablePack;

// rsolver codes as in src/main.hpp:41-47 (none 1, hlle 2, hllc 3, lhllc 4)
template <class Fn>
bool with_solver(int rsolver, Fn &&fn) {
  switch (rsolver) {
    case 1: fn(Riemann<Fluid::euler, RiemannSolver::none>()); return true;
    case 2: fn(Riemann<Fluid::euler, RiemannSolver::hlle>()); return true;
    case 3: fn(Riemann<Fluid::euler, RiemannSolver::hllc>()); return true;
    case 4: fn(Riemann<Fluid::euler, RiemannSolver::lhllc>()); return true;
  }
  return false;
}

// recon codes as in src/main.hpp:34-39 (dc 1, plm 2, ppm 3)
template <int DIR>
bool reconstruct(int recon, const parthenon::team_mbr_t &m, int k, int j, int il, int iu,
                 const VariablePack<Real> &q, ScratchPad2D<Real> &ql, ScratchPad2D<Real> &qr) {
  switch (recon) {
    case 1: Reconstruct<Reconstruction::dc, DIR>(m, k, j, il, iu, q, ql, qr); return true;
    case 2: Reconstruct<Reconstruction::plm, DIR>(m, k, j, il, iu, q, ql, qr); return true;
    case 3: Reconstruct<Reconstruction::ppm, DIR>(m, k, j, il, iu, q, ql, qr); return true;
  }
  return false;
}

}  // namespace

extern "C" {

// PLM (plm_simple.hpp:15-32) of n stencils q[s*3 + 0..2] = (q_{i-1}, q_i, q_{i+1}):
// out[s*2] = ql_{i+1}, out[s*2+1] = qr_i.
void ref_plm(const double *q, double *out, long n) {
  for (long s = 0; s < n; ++s) PLM(q[3 * s], q[3 * s + 1], q[3 * s + 2], out[2 * s], out[2 * s + 1]);
}

// PPM (ppm_simple.hpp:32-161) of n stencils q[s*5 + 0..4] = (q_{i-2} .. q_{i+2}).
void ref_ppm(const double *q, double *out, long n) {
  for (long s = 0; s < n; ++s)
    PPM(q[5 * s], q[5 * s + 1], q[5 * s + 2], q[5 * s + 3], q[5 * s + 4], out[2 * s], out[2 * s + 1]);
}

// Riemann<euler, rsolver>::Solve over n faces along direction ivx (1..3): wl, wr are (5, n)
// primitive states in the pack's variable order (rho, v1, v2, v3, p), gl, gr (2, n) the
// face values of (gamma_c, gamma_e); flx receives the (5, n) fluxes in the same order.
// Returns 0, or -1 for an unknown solver.
int ref_riemann(int rsolver, int ivx, const double *wl, const double *wr, const double *gl,
                const double *gr, double *flx, int n) {
  std::vector<double> bl(wl, wl + 5 * n), br(wr, wr + 5 * n), fl(gl, gl + 2 * n),
      fr(gr, gr + 2 * n), lam(3 * n, 0.0);
  ScratchPad2D<Real> WL(bl.data(), 5, n), WR(br.data(), 5, n), IFL(fl.data(), 2, n),
      IFR(fr.data(), 2, n);
  VariableFluxPack<Real> cons;
  cons.dim[1] = n;
  cons.dim[2] = 1;
  cons.dim[3] = 1;
  cons.dim[4] = 5;
  cons.fx[ivx - 1] = flx;
  VariablePack<Real> eos_lambda(lam.data(), 3, 1, 1, n);
  const EOS_t eos{};
  const parthenon::team_mbr_t member;
  const bool ok = with_solver(rsolver, [&](auto solver) {
    solver.Solve(member, 0, 0, 0, n - 1, ivx, WL, WR, cons, IFL, IFR, eos, eos_lambda);
  });
  return ok ? 0 : -1;
}

// The x1 face fluxes of one 1D block as CalculateFluxes computes them (hydro.cpp:580-616):
// prim (nvar, ni) and gamma (2, ni) with ni = nx + 2 ng; Reconstruct<recon, X1DIR> over
// cells ng-1 .. ng+nx of prim and gamma, Riemann::Solve over faces ng .. ng+nx, then the
// passive scalars upwinded by the mass flux.  flux (nvar, ni) receives those faces (others
// untouched).  Returns 0, or -1 for an unknown method.
int ref_x1_fluxes(int recon, int rsolver, int nvar, int nx, int ng, const double *prim,
                  const double *gamma, double *flux) {
  const int ni = nx + 2 * ng;
  // scratch one wider than the block: Reconstruct writes ql(n, i + 1) up to i = ng + nx
  std::vector<double> wl(nvar * (ni + 1)), wr(nvar * (ni + 1)), ifl(2 * (ni + 1)),
      ifr(2 * (ni + 1)), lam(3 * ni, 0.0);
  std::vector<double> q(prim, prim + (long)nvar * ni), g(gamma, gamma + 2L * ni);
  ScratchPad2D<Real> WL(wl.data(), nvar, ni + 1), WR(wr.data(), nvar, ni + 1),
      IFL(ifl.data(), 2, ni + 1), IFR(ifr.data(), 2, ni + 1);
  VariablePack<Real> P(q.data(), nvar, 1, 1, ni), G(g.data(), 2, 1, 1, ni);
  VariableFluxPack<Real> cons;
  cons.dim[1] = ni;
  cons.dim[2] = 1;
  cons.dim[3] = 1;
  cons.dim[4] = nvar;
  cons.fx[0] = flux;
  VariablePack<Real> eos_lambda(lam.data(), 3, 1, 1, ni);
  const EOS_t eos{};
  const parthenon::team_mbr_t member;
  const int is = ng, ie = ng + nx - 1;
  if (!reconstruct<parthenon::X1DIR>(recon, member, 0, 0, is - 1, ie + 1, P, WL, WR)) return -1;
  reconstruct<parthenon::X1DIR>(recon, member, 0, 0, is - 1, ie + 1, G, IFL, IFR);
  const bool ok = with_solver(rsolver, [&](auto solver) {
    solver.Solve(member, 0, 0, is, ie + 1, IV1, WL, WR, cons, IFL, IFR, eos, eos_lambda);
  });
  if (!ok) return -1;
  for (int n = NHYDRO; n < nvar; ++n)
    for (int i = is; i <= ie + 1; ++i)
      cons.flux(IV1, n, 0, 0, i) =
          cons.flux(IV1, IDN, 0, 0, i) * (cons.flux(IV1, IDN, 0, 0, i) >= 0.0 ? WL(n, i) : WR(n, i));
  return 0;
}

}  // extern "C"
