// aph_apophis.hpp -- the C++ face of the hydro path, with the names and argument meanings of
// the apophis hydro package (src/hydro/hydro.hpp:17-60, src/main.hpp:27-53), over the plain
// C ABI of aph_hydro.h.  Header-only; link libaph_hydro.so.
//
// The reference's functions take Parthenon's MeshData<Real>; here MeshData is a pack of
// meshblocks resident on the device (an aph_pack plus the stream its work goes to).  Where
// the reference aborts (PARTHENON_FAIL / PARTHENON_REQUIRE), these functions throw
// apophis_gb300::Error carrying the library's status and message; CalculateFluxes returns
// TaskStatus::complete as the reference's task does.
#ifndef APH_APOPHIS_HPP_
#define APH_APOPHIS_HPP_

#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "aph_hydro.h"

namespace apophis_gb300 {

using Real = double;

// src/main.hpp:27-53 (same numbering as the C ABI's APH_* constants)
enum class Fluid { undefined, euler };
enum class Reconstruction { undefined, dc, plm, ppm };
enum class RiemannSolver { undefined, none, hlle, hllc, lhllc };
enum class Integrator { undefined, rk1, rk2, rk3, vl2 };
enum class TaskStatus { fail, complete };

class Error : public std::runtime_error {
 public:
  Error(aph_status status, const std::string &what)
      : std::runtime_error(what + ": " + aph_last_error()), status(status) {}
  aph_status status;
};

inline void check(aph_status st, const char *what) {
  if (st != APH_OK) throw Error(st, what);
}

// A pack of meshblocks (Parthenon's MeshData<Real> of one partition): the blocks' device
// fields (aph_block), the hydro parameters, the block grid and its physical boundaries.
class MeshData {
 public:
  MeshData(const aph_hydro_params &params, const std::vector<aph_block> &blocks, const int nb[3],
           const int bc[6], void *stream = nullptr)
      : params_(params), blocks_(blocks), stream_(stream) {
    check(aph_pack_create(&params_, blocks_.data(), (int)blocks_.size(), &pack_), "aph_pack_create");
    const aph_status st = aph_pack_set_topology(pack_, nb, bc);
    if (st != APH_OK) {
      aph_pack_destroy(pack_);
      throw Error(st, "aph_pack_set_topology");
    }
  }
  ~MeshData() { aph_pack_destroy(pack_); }
  MeshData(const MeshData &) = delete;
  MeshData &operator=(const MeshData &) = delete;

  aph_pack pack() const { return pack_; }
  void *stream() const { return stream_; }
  const aph_hydro_params &params() const { return params_; }
  int NumBlocks() const { return (int)blocks_.size(); }

 private:
  aph_hydro_params params_;
  std::vector<aph_block> blocks_;
  void *stream_;
  aph_pack pack_ = nullptr;
};

// ConsToPrim<EOS_t> (hydro.cpp:422-533), registered as FillDerivedMesh.
template <class EOS>
void ConsToPrim(MeshData *md) {
  check(aph_hydro_cons_to_prim(md->pack(), md->stream()), "ConsToPrim");
}

// CalculateFluxes<fluid, recon, rsolver> (hydro.cpp:535-744), the flux task.
template <Fluid fluid, Reconstruction recon, RiemannSolver rsolver>
TaskStatus CalculateFluxes(std::shared_ptr<MeshData> &md) {
  static_assert(fluid == Fluid::euler, "the hydro path implements the Euler fluid");
  check(aph_hydro_calculate_fluxes(md->pack(), (int)recon, (int)rsolver, md->stream()),
        "CalculateFluxes");
  return TaskStatus::complete;
}

// The runtime-dispatched form (hydro.cpp:114-139 selects the template from the parameters).
inline TaskStatus CalculateFluxes(std::shared_ptr<MeshData> &md) {
  const aph_hydro_params &p = md->params();
  check(aph_hydro_calculate_fluxes(md->pack(), p.recon, p.rsolver, md->stream()), "CalculateFluxes");
  return TaskStatus::complete;
}

// EstimateTimestep<fluid> (hydro.cpp:351-420), registered as EstimateTimestepMesh.
template <Fluid fluid>
Real EstimateTimestep(MeshData *md) {
  static_assert(fluid == Fluid::euler, "the hydro path implements the Euler fluid");
  double dt = 0.0;
  check(aph_hydro_estimate_timestep(md->pack(), &dt, md->stream()), "EstimateTimestep");
  return dt;
}

// Parthenon's UpdateWithFluxDivergence(u0, u1, gam0, gam1, beta_dt) (apophis_driver.cpp:79-82):
// u0 <- gam0 u0 + gam1 u1 - beta_dt div F over the interior; the pack's blocks carry u1.
inline TaskStatus UpdateWithFluxDivergence(MeshData *md, Real gam0, Real gam1, Real beta_dt) {
  check(aph_hydro_update_with_flux_divergence(md->pack(), gam0, gam1, beta_dt, md->stream()),
        "UpdateWithFluxDivergence");
  return TaskStatus::complete;
}

// Ghost exchange and ApplyBoundaryConditions (apophis_driver.cpp:94-104).
inline TaskStatus FillGhosts(MeshData *md) {
  check(aph_hydro_fill_ghosts(md->pack(), md->stream()), "FillGhosts");
  return TaskStatus::complete;
}

// ApplyGravity, constant g (gravity.cpp:374-410).
inline TaskStatus ApplyGravity(MeshData *md, const Real g[3], Real beta_dt) {
  check(aph_hydro_apply_gravity(md->pack(), g, beta_dt, md->stream()), "ApplyGravity");
  return TaskStatus::complete;
}

// GlobalQuantHst<Sum, idx> (hydro.cpp:754-771): idx 0 (IDN) total mass, 4 (IEN) total energy.
template <int idx>
Real GlobalQuantHst(MeshData *md) {
  static_assert(idx == 0 || idx == 4, "the history sums are of IDN and IEN");
  double out[2];
  check(aph_hydro_history(md->pack(), out, md->stream()), "GlobalQuantHst");
  return idx == 0 ? out[0] : out[1];
}

}  // namespace apophis_gb300

#endif  // APH_APOPHIS_HPP_
