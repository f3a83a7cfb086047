"""apophis_gb300: a GB300-native (sm_103a) implementation of apophis's hydro flux path.

ConsToPrim (ideal gas) -> PLM/PPM reconstruction -> HLLE/HLLC fluxes per sweep ->
flux-divergence Runge-Kutta stage update -> CFL timestep min-reduction, as hand-written
CUDA kernels behind the C ABI declared in include/aph_hydro.h.
"""
from .mesh import MeshConfig  # noqa: F401
