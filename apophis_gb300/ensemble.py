"""Ensembles: independent 2D problems batched in one pack and stepped by one persistent
launch per RK stage (aph_ensemble in include/aph_hydro.h).

Each member is a uniform periodic (or walled) 2D mesh of equal meshblocks with its own
adiabatic index, CFL dt, clock and end time.  The pack concatenates the members' blocks in
order; block b of member m keeps the uniform pack's x-fastest numbering, and its face table
names neighbours inside the member only.

``blast_ensemble`` builds the batched blast-wave workload: 64 members with grids drawn from
{128, 192, 256, 384, 512}^2 (blocks of 64^2), gamma ~ U[1.4, 5/3], rho = 1, p = 10 inside a
radius r0 ~ U[0.05, 0.15] of the box centre and 0.1 outside, periodic, PPM + HLLC, RK2, to
t = 0.1.
"""
import ctypes
from dataclasses import dataclass
from typing import List

import numpy as np

from . import amr, problems
from .mesh import MeshConfig
from .stepper import Stepper as _StepperBase


@dataclass
class Ensemble:
    members: List[MeshConfig]
    tlim: List[float]

    def __post_init__(self):
        self.mesh = []         # per member: the unrefined AmrConfig of its blocks
        self.block0 = []       # per member: its first block in the pack
        self.offset = []       # per block: first cell (entire domain) in the flat pack
        self.member_of = []
        nb = 0
        off = 0
        for m, cfg in enumerate(self.members):
            if cfg.ndim != 2:
                raise ValueError("ensemble members are 2D meshes")
            ac = amr.uniform_as_amr(cfg)
            self.mesh.append(ac)
            self.block0.append(nb)
            for b in range(ac.nblocks):
                self.offset.append(off + ac.offset[b])
                self.member_of.append(m)
            nb += ac.nblocks
            off += ac.total_cells
        self.nblocks = nb
        self.total_cells = off
        first = self.members[0]
        for cfg in self.members:
            for attr in ("ng", "recon", "rsolver", "integrator", "cfl", "dfloor", "pfloor", "nscalars"):
                if getattr(cfg, attr) != getattr(first, attr):
                    raise ValueError("ensemble members share %s" % attr)

    @property
    def nmembers(self):
        return len(self.members)

    @property
    def nvar(self):
        return self.members[0].nvar

    def zones(self):
        return sum(c.zones() for c in self.members)

    def member_slice(self, m):
        """Slice of the flat pack (nvar values per cell) holding member m."""
        start = self.nvar * self.offset[self.block0[m]]
        return slice(start, start + self.nvar * self.mesh[m].total_cells)

    def pack(self, conses):
        """Flat pack from the members' (nblocks, nvar, nk, nj, ni) arrays."""
        out = np.empty(self.nvar * self.total_cells)
        for m, c in enumerate(conses):
            out[self.member_slice(m)] = np.ascontiguousarray(c).reshape(-1)
        return out

    def unpack(self, flat, m):
        return flat[self.member_slice(m)].reshape(self.members[m].pack_shape(self.nvar))

    def blocks(self):
        """(AmrBlock with pack-wide neighbour indices, member) per block."""
        out = []
        for m, ac in enumerate(self.mesh):
            b0 = self.block0[m]
            for B in ac.blocks:
                C = amr.AmrBlock(B.level, B.origin, B.nx, B.dx, list(B.face_kind),
                                 [[b0 + n for n in nbrs] for nbrs in B.face_nbr])
                out.append(C)
        return out


def blast_ensemble(nmembers=64, seed=0, sizes=(128, 192, 256, 384, 512), block=64, ng=4,
                   recon="ppm", rsolver="hllc", integrator="rk2", cfl=0.3, tlim=0.1):
    """The batched blast-wave workload (seeded numpy PCG64): returns (Ensemble, flat cons)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    cfgs, conses = [], []
    for m in range(nmembers):
        n = int(sizes[rng.integers(len(sizes))])
        gamma = float(rng.uniform(1.4, 5.0 / 3.0))
        r0 = float(rng.uniform(0.05, 0.15))
        cfg, cons = problems.blast2d(n=n, block=min(block, n), ng=ng, r0=r0, gamma=gamma,
                                     recon=recon, rsolver=rsolver, integrator=integrator, cfl=cfl)
        cfg.name = "blast2d_m%d" % m
        cfgs.append(cfg)
        conses.append(cons)
    ens = Ensemble(cfgs, [tlim] * nmembers)
    return ens, ens.pack(conses)


class EnsembleStepper(_StepperBase):
    """All members in one stepper: one persistent launch per stage over every block, each
    member with its own gas constants, dt and clock (finished members are skipped)."""

    def interior_values(self):
        return self.ens.nvar * sum(c.zones() for c in self.ens.members)

    def __init__(self, ens: Ensemble, cons0, exact=True, fixed_dt=0.0):
        import torch
        from . import _capi
        from .hydro import require_cuda
        require_cuda()
        _capi.load()
        self.ens = ens
        self.cfg = ens.members[0]
        self.exact = exact
        nv = ens.nvar
        self.cons = torch.zeros(nv * ens.total_cells, dtype=torch.float64, device="cuda")
        self.cons.copy_(torch.as_tensor(np.ascontiguousarray(cons0)))
        nb = ens.nblocks
        blks = ens.blocks()
        blocks = (_capi.aph_block * nb)()
        for b, B in enumerate(blks):
            blocks[b].cons = self.cons.data_ptr() + 8 * nv * ens.offset[b]
            blocks[b].nx[:] = [B.nx[0], B.nx[1], 1]
            blocks[b].dx[:] = [B.dx[0], B.dx[1], 1.0]
        table = self.face_table(blks)
        self._member = (ctypes.c_int * nb)(*ens.member_of)
        self._gm1 = (ctypes.c_double * ens.nmembers)(*[c.gm1 for c in ens.members])
        self._tlim = (ctypes.c_double * ens.nmembers)(*ens.tlim)
        self._ens = _capi.aph_ensemble(ens.nmembers, self._member, self._gm1, self._tlim)
        self._blocks, self._table = blocks, table
        c0 = ens.members[0]
        desc = _capi.aph_stepper_desc()
        desc.params = _capi.aph_hydro_params(2, c0.ng, nv, _capi.RECON[c0.recon],
                                             _capi.RSOLVER[c0.rsolver], c0.gm1, c0.dfloor,
                                             c0.pfloor, c0.cfl, 1 if exact else 0)
        desc.integrator = _capi.INTEGRATOR[c0.integrator]
        desc.nblocks = nb
        desc.blocks = ctypes.cast(blocks, ctypes.POINTER(_capi.aph_block))
        desc.nb[:] = [nb, 1, 1]
        desc.bc[:] = [_capi.BC[c0.bc[d][s]] for d in range(2) for s in range(2)] + [0, 0]
        desc.use_gravity = 0
        desc.tlim = 0.0
        desc.fixed_dt = fixed_dt
        desc.amr = ctypes.cast(table, ctypes.POINTER(_capi.aph_amr_block))
        desc.ensemble = ctypes.pointer(self._ens)
        self.h = ctypes.c_void_p()
        _capi.call("aph_stepper_create", ctypes.byref(desc), ctypes.byref(self.h))

    @staticmethod
    def face_table(blks):
        from . import _capi
        table = (_capi.aph_amr_block * len(blks))()
        for b, B in enumerate(blks):
            t = table[b]
            t.level = B.level
            t.origin[0], t.origin[1] = B.origin
            for f in range(4):
                t.face_kind[f] = B.face_kind[f]
                t.face_count[f] = len(B.face_nbr[f])
                for k, x in enumerate(B.face_nbr[f]):
                    t.face_nbr[f][k] = x
        return table

    def member_status(self):
        from . import _capi
        from .hydro import stream_handle
        n = self.ens.nmembers
        t, dt, cyc = (ctypes.c_double * n)(), (ctypes.c_double * n)(), (ctypes.c_int * n)()
        _capi.call("aph_stepper_member_status", self.h, t, dt, cyc, stream_handle())
        return {"time": list(t), "dt": list(dt), "ncycle": list(cyc)}

    def run_to_end(self, chunk=8, max_steps=100000):
        """Step until every member reaches its end time; returns the steps launched."""
        done = 0
        while done < max_steps:
            self.step(chunk)
            done += chunk
            if self.status()["dt"] == 0.0:
                break
        return done

    def tune_key(self):
        import torch
        e = self.ens
        sizes = ",".join("%dx%d" % tuple(c.mesh_nx[:2]) for c in e.members)
        return "%s|ensemble|members%d|blocks%d|%s|%s|%s|%s|exact%d" % (
            torch.cuda.get_device_name(), e.nmembers, e.nblocks, sizes, e.members[0].recon,
            e.members[0].rsolver, e.members[0].integrator, int(self.exact))
