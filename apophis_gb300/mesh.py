"""Mesh and meshblock geometry for the hydro path.

A mesh is a uniform grid of equal meshblocks (Parthenon's ``<parthenon/mesh>`` and
``<parthenon/meshblock>`` blocks).  Each meshblock stores a field as
``(nvar, nk, nj, ni)`` with ``i`` fastest and ``ng`` ghost cells on each side of
every active dimension (Parthenon's ``VariablePack(b, n, k, j, i)``, used at
src/hydro/hydro.cpp:453-469); a pack of blocks is ``(nblocks, nvar, nk, nj, ni)``.
Blocks are numbered x-fastest: ``b = (bk * nb2 + bj) * nb1 + bi``.
"""
from dataclasses import dataclass, field
from typing import Optional, Tuple

import numpy as np

# Variable indices: src/main.hpp:6-20
IDN, IM1, IM2, IM3, IEN = 0, 1, 2, 3, 4
IV1, IV2, IV3, IPR = 1, 2, 3, 4
NHYDRO = 5

# Default floors: sqrt(1024 * FLT_MIN) = 2**-58 (src/hydro/hydro.cpp:295-296)
DEFAULT_FLOOR = float(np.sqrt(1024.0 * float(np.finfo(np.float32).tiny)))

# Ghost cells each reconstruction needs: src/hydro/hydro.cpp:56-75
RECON_NEED_GHOST = {"dc": 1, "plm": 2, "ppm": 3}


@dataclass
class MeshConfig:
    ndim: int
    mesh_nx: Tuple[int, int, int]
    block_nx: Tuple[int, int, int]
    ng: int
    xmin: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    xmax: Tuple[float, float, float] = (1.0, 1.0, 1.0)
    bc: Tuple[Tuple[str, str], ...] = (("periodic", "periodic"),) * 3
    recon: str = "ppm"
    rsolver: str = "hllc"
    integrator: str = "rk2"
    gamma: float = 1.4
    cfl: float = 0.3
    dfloor: float = DEFAULT_FLOOR
    pfloor: float = DEFAULT_FLOOR
    gravity: Optional[Tuple[float, float, float]] = None
    name: str = field(default="mesh")
    nscalars: int = 0   # passive scalars (hydro/composition), conserved as rho * s

    def __post_init__(self):
        self.mesh_nx = tuple(int(x) for x in self.mesh_nx)
        self.block_nx = tuple(int(x) for x in self.block_nx)
        for d in range(3):
            if d >= self.ndim and (self.mesh_nx[d] != 1 or self.block_nx[d] != 1):
                raise ValueError("unused dimension %d must have one cell" % (d + 1))
            if self.mesh_nx[d] % self.block_nx[d]:
                raise ValueError("mesh nx%d not a multiple of meshblock nx%d" % (d + 1, d + 1))
        if self.ng < RECON_NEED_GHOST[self.recon]:
            raise ValueError("Not enough ghost zones for reconstruction")

    @property
    def gm1(self):
        return self.gamma - 1.0

    @property
    def nvar(self):
        return NHYDRO + self.nscalars

    @property
    def blocks_per_dim(self):
        return tuple(self.mesh_nx[d] // self.block_nx[d] for d in range(3))

    @property
    def nblocks(self):
        b = self.blocks_per_dim
        return b[0] * b[1] * b[2]

    @property
    def dx(self):
        return tuple((self.xmax[d] - self.xmin[d]) / self.mesh_nx[d] for d in range(3))

    @property
    def entire(self):
        """(ni, nj, nk) of one meshblock, ghosts included."""
        ni = self.block_nx[0] + 2 * self.ng
        nj = self.block_nx[1] + 2 * self.ng if self.ndim >= 2 else 1
        nk = self.block_nx[2] + 2 * self.ng if self.ndim >= 3 else 1
        return ni, nj, nk

    def pack_shape(self, nvar=NHYDRO):
        ni, nj, nk = self.entire
        return (self.nblocks, nvar, nk, nj, ni)

    @property
    def interior(self):
        """Slices (k, j, i) of the interior of a meshblock."""
        g = self.ng
        ni, nj, nk = self.entire
        si = slice(g, ni - g)
        sj = slice(g, nj - g) if self.ndim >= 2 else slice(0, 1)
        sk = slice(g, nk - g) if self.ndim >= 3 else slice(0, 1)
        return sk, sj, si

    def block_index(self, b):
        nb = self.blocks_per_dim
        return b % nb[0], (b // nb[0]) % nb[1], b // (nb[0] * nb[1])

    def cell_centers(self, b):
        """Interior cell-centre coordinates (x, y, z) of block b, each shaped (nk, nj, ni)."""
        bi, bj, bk = self.block_index(b)
        dx = self.dx
        bn = self.block_nx
        xs = []
        for d, bd in enumerate((bi, bj, bk)):
            idx = bd * bn[d] + np.arange(bn[d]) + 0.5
            xs.append(self.xmin[d] + idx * dx[d])
        z, y, x = np.meshgrid(xs[2], xs[1], xs[0], indexing="ij")
        return x, y, z

    def zones(self):
        return self.mesh_nx[0] * self.mesh_nx[1] * self.mesh_nx[2]

    def to_global(self, pack):
        """Interior of a pack (nblocks, nvar, ...) assembled to (nvar, NZ, NY, NX)."""
        nvar = pack.shape[1]
        nb = self.blocks_per_dim
        bn = self.block_nx
        out = np.empty((nvar, self.mesh_nx[2], self.mesh_nx[1], self.mesh_nx[0]), pack.dtype)
        sk, sj, si = self.interior
        for b in range(self.nblocks):
            bi, bj, bk = self.block_index(b)
            out[:, bk * bn[2]:(bk + 1) * bn[2], bj * bn[1]:(bj + 1) * bn[1],
                bi * bn[0]:(bi + 1) * bn[0]] = pack[b][:, sk, sj, si]
        return out
