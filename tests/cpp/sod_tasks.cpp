// A host program in the reference's terms: the Sod shock tube advanced through the C++ face
// of the library (aph_apophis.hpp) in the stage order of ApophisDriver::MakeTaskCollection
// (src/apophis_driver.cpp:27-129): u1 <- u0, CalculateFluxes, UpdateWithFluxDivergence,
// FillGhosts (boundary exchange + conditions), ConsToPrim (FillDerived), and the dt policy
// dt_{n+1} = min(2 dt_n, EstimateTimestep) clipped at tlim.
//
// usage: sod_tasks <initial cons file> <final cons file> <nx> <tlim> <exact 0|1>
// Files are raw float64: (5, nx + 2 nghost) cons; the output adds time and cycle count.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <vector>

#include "aph_apophis.hpp"

using namespace apophis_gb300;

struct IdealGas {};

int main(int argc, char **argv) {
  if (argc != 6) {
    std::fprintf(stderr, "usage: %s in.bin out.bin nx tlim exact\n", argv[0]);
    return 2;
  }
  const int nx = std::atoi(argv[3]), ng = 2;
  const double tlim = std::atof(argv[4]);
  const int exact = std::atoi(argv[5]);
  const int ni = nx + 2 * ng;
  std::vector<double> cons(5 * ni);
  FILE *f = std::fopen(argv[1], "rb");
  if (!f || std::fread(cons.data(), sizeof(double), cons.size(), f) != cons.size()) return 3;
  std::fclose(f);

  double *d_cons, *d_u1, *d_prim, *d_gamma, *d_flux;
  const size_t bytes = cons.size() * sizeof(double);
  if (cudaMalloc(&d_cons, bytes) || cudaMalloc(&d_u1, bytes) || cudaMalloc(&d_prim, bytes) ||
      cudaMalloc(&d_gamma, 2 * ni * sizeof(double)) || cudaMalloc(&d_flux, bytes))
    return 4;
  cudaMemcpy(d_cons, cons.data(), bytes, cudaMemcpyHostToDevice);

  aph_hydro_params p{};
  p.ndim = 1;
  p.nghost = ng;
  p.nvar = 5;
  p.recon = (int)Reconstruction::plm;
  p.rsolver = (int)RiemannSolver::hlle;
  p.gm1 = 1.4 - 1.0;  // gamma - 1 as the problem setup computes it
  p.dfloor = std::ldexp(1.0, -58);
  p.pfloor = std::ldexp(1.0, -58);
  p.cfl = 0.4;
  p.exact = exact;
  aph_block b{};
  b.cons = d_cons;
  b.prim = d_prim;
  b.gamma = d_gamma;
  b.u1 = d_u1;
  b.flux[0] = d_flux;
  b.nx[0] = nx;
  b.nx[1] = b.nx[2] = 1;
  b.dx[0] = 1.0 / nx;
  b.dx[1] = b.dx[2] = 1.0;
  const int nb[3] = {1, 1, 1};
  const int bc[6] = {APH_BC_OUTFLOW, APH_BC_OUTFLOW, APH_BC_PERIODIC, APH_BC_PERIODIC,
                     APH_BC_PERIODIC, APH_BC_PERIODIC};
  try {
    auto md = std::make_shared<MeshData>(p, std::vector<aph_block>{b}, nb, bc);
    FillGhosts(md.get());
    ConsToPrim<IdealGas>(md.get());
    double dt = EstimateTimestep<Fluid::euler>(md.get());
    double time = 0.0;
    int ncycle = 0;
    const double stages[2][3] = {{0.0, 1.0, 1.0}, {0.5, 0.5, 0.5}};  // RK2 (gam0, gam1, beta)
    while (time < tlim) {
      if (tlim - time < dt) dt = tlim - time;
      for (int s = 0; s < 2; ++s) {
        if (s == 0) cudaMemcpy(d_u1, d_cons, bytes, cudaMemcpyDeviceToDevice);
        CalculateFluxes<Fluid::euler, Reconstruction::plm, RiemannSolver::hlle>(md);
        UpdateWithFluxDivergence(md.get(), stages[s][0], stages[s][1], stages[s][2] * dt);
        FillGhosts(md.get());
        ConsToPrim<IdealGas>(md.get());
      }
      time += dt;
      ++ncycle;
      const double est = EstimateTimestep<Fluid::euler>(md.get());
      dt = est < 2.0 * dt ? est : 2.0 * dt;
    }
    const double mass = GlobalQuantHst<0>(md.get());
    cudaMemcpy(cons.data(), d_cons, bytes, cudaMemcpyDeviceToHost);
    FILE *o = std::fopen(argv[2], "wb");
    std::fwrite(cons.data(), sizeof(double), cons.size(), o);
    const double tail[3] = {time, (double)ncycle, mass};
    std::fwrite(tail, sizeof(double), 3, o);
    std::fclose(o);
  } catch (const Error &e) {
    std::fprintf(stderr, "error %d: %s\n", e.status, e.what());
    return 5;
  }
  cudaFree(d_cons);
  cudaFree(d_u1);
  cudaFree(d_prim);
  cudaFree(d_gamma);
  cudaFree(d_flux);
  return 0;
}
