"""Statically refined 2D meshes of uneven meshblocks.

A mesh is a list of leaf meshblocks, each at a refinement level l (cell width dx0 / 2^l),
with its own cell count per side and the global index (in cells of its level) of its first
interior cell.  ``face table``: for each face (x-, x+, y-, y+) the kind of neighbour --
SAME level, COARSER (one block), FINER (the blocks that cover the face, in transverse
order), or BOUNDARY (a physical outflow / reflecting boundary; periodic faces point at the
wrapped neighbour) -- and the neighbour indices.  Levels differ by at most one across a
face.  The pack is stored flat: block b's fields start at ``offset[b]`` cells x nvar.

``rt2d_amr`` builds the Rayleigh-Taylor configuration: a 256 x 768 base grid of 32^2
blocks on [0,0.5]x[0,1.5] with two static refinement levels of 16^2 blocks around the
interface (about 1,400 blocks).
"""
import ctypes
import math
from dataclasses import dataclass, field
from typing import List, Optional, Tuple

import numpy as np

from .mesh import DEFAULT_FLOOR, IDN, IEN, IM1, IM2, IM3, RECON_NEED_GHOST
from .stepper import Stepper as _StepperBase

FACE_SAME, FACE_COARSER, FACE_FINER, FACE_BOUNDARY = 0, 1, 2, 3


@dataclass
class AmrBlock:
    level: int
    origin: Tuple[int, int]   # global index of the first interior cell, in cells of its level
    nx: Tuple[int, int]
    dx: Tuple[float, float]
    face_kind: List[int] = field(default_factory=lambda: [FACE_BOUNDARY] * 4)
    face_nbr: List[List[int]] = field(default_factory=lambda: [[] for _ in range(4)])


@dataclass
class AmrConfig:
    blocks: List[AmrBlock]
    ng: int
    base_nx: Tuple[int, int]
    xmin: Tuple[float, float]
    xmax: Tuple[float, float]
    bc: Tuple[Tuple[str, str], Tuple[str, str]]
    recon: str = "ppm"
    rsolver: str = "hllc"
    integrator: str = "rk2"
    gamma: float = 1.4
    cfl: float = 0.4
    dfloor: float = DEFAULT_FLOOR
    pfloor: float = DEFAULT_FLOOR
    gravity: Optional[Tuple[float, float, float]] = None
    name: str = "amr"
    ndim: int = 2
    nscalars: int = 0   # passive scalars (hydro/composition), conserved as rho * s

    def __post_init__(self):
        if self.ng < RECON_NEED_GHOST[self.recon]:
            raise ValueError("Not enough ghost zones for reconstruction")
        self.offset = []
        off = 0
        for B in self.blocks:
            self.offset.append(off)
            off += self.entire(B)[0] * self.entire(B)[1]
        self.total_cells = off

    @property
    def gm1(self):
        return self.gamma - 1.0

    @property
    def nvar(self):
        return 5 + self.nscalars

    @property
    def nblocks(self):
        return len(self.blocks)

    def entire(self, B):
        return B.nx[0] + 2 * self.ng, B.nx[1] + 2 * self.ng

    def zones(self):
        return sum(B.nx[0] * B.nx[1] for B in self.blocks)

    def flat_size(self, nvar=None):
        return (self.nvar if nvar is None else nvar) * self.total_cells

    def block_view(self, flat, b, nvar=None):
        """(nvar, 1, nj, ni) view of block b in a flat pack."""
        nvar = self.nvar if nvar is None else nvar
        ni, nj = self.entire(self.blocks[b])
        o = self.offset[b] * nvar
        return flat[o:o + nvar * ni * nj].reshape(nvar, 1, nj, ni)

    def cell_centers(self, b):
        B = self.blocks[b]
        xs = [self.xmin[d] + (B.origin[d] + np.arange(B.nx[d]) + 0.5) * B.dx[d] for d in range(2)]
        y, x = np.meshgrid(xs[1], xs[0], indexing="ij")
        return x, y

    def level_counts(self):
        out = {}
        for B in self.blocks:
            out[B.level] = out.get(B.level, 0) + 1
        return out


def build(base_nx, block0, blockf, levels, xmin, xmax, bc, refine):
    """Leaf blocks of a static refinement.  refine(level, x0, y0, x1, y1) -> True refines the
    block covering [x0,x1]x[y0,y1] to the next level (up to `levels` extra levels).  Level-0
    blocks have block0 cells per side, finer levels blockf."""
    dx0 = tuple((xmax[d] - xmin[d]) / base_nx[d] for d in range(2))
    leaves = []

    def add(level, origin, n):
        dx = (dx0[0] / 2 ** level, dx0[1] / 2 ** level)
        x0 = xmin[0] + origin[0] * dx[0]
        y0 = xmin[1] + origin[1] * dx[1]
        x1, y1 = x0 + n * dx[0], y0 + n * dx[1]
        if level < levels and refine(level, x0, y0, x1, y1):
            # children cover the same region with blockf-cell blocks at level+1
            m = 2 * n // blockf
            for cj in range(m):
                for ci in range(m):
                    add(level + 1, (2 * origin[0] + ci * blockf, 2 * origin[1] + cj * blockf), blockf)
        else:
            leaves.append(AmrBlock(level, origin, (n, n), dx))

    for bj in range(base_nx[1] // block0):
        for bi in range(base_nx[0] // block0):
            add(0, (bi * block0, bj * block0), block0)
    _link(leaves, base_nx, bc)
    return leaves


def _link(leaves, base_nx, bc):
    levels = max(B.level for B in leaves) + 1
    owner = []
    for l in range(levels):
        owner.append(-np.ones((base_nx[1] << l, base_nx[0] << l), dtype=np.int64))
    for b, B in enumerate(leaves):
        owner[B.level][B.origin[1]:B.origin[1] + B.nx[1], B.origin[0]:B.origin[0] + B.nx[0]] = b
    for b, B in enumerate(leaves):
        l = B.level
        for d in range(2):
            t = 1 - d
            N = (base_nx[0] << l, base_nx[1] << l)
            for s in range(2):
                face = 2 * d + s
                g = B.origin[d] - 1 if s == 0 else B.origin[d] + B.nx[d]
                if g < 0 or g >= N[d]:
                    if bc[d][s] != "periodic":
                        B.face_kind[face] = FACE_BOUNDARY
                        B.face_nbr[face] = []
                        continue
                    g %= N[d]
                tr = range(B.origin[t], B.origin[t] + B.nx[t])

                def at(level, gd, gt):
                    idx = [0, 0]
                    idx[d], idx[t] = gd, gt
                    return int(owner[level][idx[1], idx[0]])

                same = {at(l, g, x) for x in tr}
                if -1 not in same:
                    assert len(same) == 1, "same-level neighbour must cover the whole face"
                    B.face_kind[face] = FACE_SAME
                    B.face_nbr[face] = [same.pop()]
                    continue
                if l > 0:
                    coarse = {at(l - 1, g >> 1, x >> 1) for x in tr}
                    if -1 not in coarse:
                        assert len(coarse) == 1
                        B.face_kind[face] = FACE_COARSER
                        B.face_nbr[face] = [coarse.pop()]
                        continue
                assert l + 1 < levels, "neighbour differs by more than one level"
                gf = 2 * g + (1 if s == 0 else 0)  # fine cell adjacent to the face
                fine = []
                for x in range(2 * tr.start, 2 * tr.stop):
                    o = at(l + 1, gf, x)
                    assert o >= 0, "neighbour differs by more than one level"
                    if not fine or fine[-1] != o:
                        fine.append(o)
                B.face_kind[face] = FACE_FINER
                B.face_nbr[face] = fine
                assert len(fine) <= 4


def rt2d_amr(nx=256, ny=768, block0=32, blockf=16, ng=4, recon="ppm", rsolver="hllc",
             integrator="rk2", cfl=0.4, gamma=1.4, g=-0.1, band1=0.125, band2=0.0625):
    """Rayleigh-Taylor on [0,0.5]x[0,1.5] (as problems.rt2d) with level 1 where the block
    is within band1 of the interface y = 0.75 and level 2 within band2."""
    xmin, xmax = (0.0, 0.0), (0.5, 1.5)
    bc = (("periodic", "periodic"), ("reflecting", "reflecting"))

    def refine(level, x0, y0, x1, y1):
        w = band1 if level == 0 else band2
        return y0 < 0.75 + w and y1 > 0.75 - w

    leaves = build((nx, ny), block0, blockf, 2, xmin, xmax, bc, refine)
    cfg = AmrConfig(leaves, ng, (nx, ny), xmin, xmax, bc, recon=recon, rsolver=rsolver,
                    integrator=integrator, gamma=gamma, cfl=cfl, gravity=(0.0, g, 0.0),
                    name="rt2d_amr")
    cons = np.zeros(cfg.flat_size(5))
    gm1 = cfg.gm1
    for b in range(cfg.nblocks):
        x, y = cfg.cell_centers(b)
        xc, yc = x - 0.25, y - 0.75
        rho = np.where(yc < 0.0, 1.0, 2.0)
        vy = 0.01 * (1.0 + np.cos(4.0 * math.pi * xc)) * (1.0 + np.cos(3.0 * math.pi * yc)) / 4.0
        p = 1.0 / gamma + g * rho * yc
        v = cfg.block_view(cons, b)
        s = (0, slice(ng, -ng), slice(ng, -ng))
        v[IDN][s] = rho
        v[IM1][s] = 0.0
        v[IM2][s] = rho * vy
        v[IM3][s] = 0.0
        v[IEN][s] = p / gm1 + 0.5 * rho * vy * vy
    return cfg, cons


def small_test_mesh(recon="ppm", rsolver="hllc", ng=4, integrator="rk2"):
    """A small two-level mesh for the parity tests: 64 x 64 base cells of 16^2 blocks on the
    periodic unit square, level 1 (16^2 blocks) in the central square, KH-like shear."""
    xmin, xmax = (0.0, 0.0), (1.0, 1.0)
    bc = (("periodic", "periodic"), ("periodic", "periodic"))

    def refine(level, x0, y0, x1, y1):
        return x0 >= 0.25 and x1 <= 0.75 and y0 >= 0.25 and y1 <= 0.75

    leaves = build((64, 64), 16, 16, 1, xmin, xmax, bc, refine)
    cfg = AmrConfig(leaves, ng, (64, 64), xmin, xmax, bc, recon=recon, rsolver=rsolver,
                    integrator=integrator, gamma=5.0 / 3.0, cfl=0.3, name="amr_small")
    cons = np.zeros(cfg.flat_size(5))
    for b in range(cfg.nblocks):
        x, y = cfg.cell_centers(b)
        band = 0.5 * (np.tanh((y - 0.3) / 0.05) - np.tanh((y - 0.7) / 0.05))
        rho = 1.0 + band + 0.05 * np.sin(2 * math.pi * (x + y) + 0.3)
        vx = band - 0.5
        vy = 0.02 * np.sin(2 * math.pi * x + 0.1)
        p = 2.5 + 0.1 * np.cos(2 * math.pi * (x - y) + 0.7)
        v = cfg.block_view(cons, b)
        s = (0, slice(ng, -ng), slice(ng, -ng))
        v[IDN][s] = rho
        v[IM1][s] = rho * vx
        v[IM2][s] = rho * vy
        v[IM3][s] = 0.0
        v[IEN][s] = p / cfg.gm1 + 0.5 * rho * (vx * vx + vy * vy)
    return cfg, cons


# ---- GPU paths over the C ABI ---------------------------------------------------------------
def amr_table(cfg):
    """ctypes array of aph_amr_block for cfg."""
    from . import _capi
    arr = (_capi.aph_amr_block * cfg.nblocks)()
    for b, B in enumerate(cfg.blocks):
        a = arr[b]
        a.level = B.level
        a.origin[0], a.origin[1] = B.origin
        for f in range(4):
            a.face_kind[f] = B.face_kind[f]
            a.face_count[f] = len(B.face_nbr[f])
            for n, nb in enumerate(B.face_nbr[f]):
                a.face_nbr[f][n] = nb
    return arr


def check_table(cfg, table=None):
    """Run the library's host-side face-table check (raises _capi.AphError)."""
    from . import _capi
    _capi.load()
    table = amr_table(cfg) if table is None else table
    nx = (ctypes.c_int * (2 * cfg.nblocks))(*[n for B in cfg.blocks for n in B.nx])
    _capi.call("aph_amr_check", table, nx, cfg.nblocks, cfg.ng)


def _bc_array(cfg):
    from . import _capi
    return (ctypes.c_int * 6)(*[_capi.BC[cfg.bc[d][s]] for d in range(2) for s in range(2)], 0, 0)


def _params(cfg, exact):
    from . import _capi
    return _capi.aph_hydro_params(2, cfg.ng, cfg.nvar, _capi.RECON[cfg.recon], _capi.RSOLVER[cfg.rsolver],
                                  cfg.gm1, cfg.dfloor, cfg.pfloor, cfg.cfl, 1 if exact else 0)


class AmrMeshData:
    """Flat device fields of a refined pack and its C-ABI pack (plus per-block partitions)."""

    def __init__(self, cfg: AmrConfig, exact=True):
        import torch
        from . import _capi
        from .hydro import require_cuda
        require_cuda()
        _capi.load()
        self.cfg = cfg
        kw = dict(dtype=torch.float64, device="cuda")
        n, nv = cfg.total_cells, cfg.nvar
        self.cons = torch.zeros(nv * n, **kw)
        self.prim = torch.zeros(nv * n, **kw)
        self.u1 = torch.zeros(nv * n, **kw)
        self.gamma = torch.zeros(2 * n, **kw)
        self.flux = [torch.zeros(nv * n, **kw), torch.zeros(nv * n, **kw)]
        blocks = (_capi.aph_block * cfg.nblocks)()
        for b, B in enumerate(cfg.blocks):
            o = cfg.offset[b]
            blk = blocks[b]
            blk.cons = self.cons.data_ptr() + 8 * nv * o
            blk.prim = self.prim.data_ptr() + 8 * nv * o
            blk.u1 = self.u1.data_ptr() + 8 * nv * o
            blk.gamma = self.gamma.data_ptr() + 8 * 2 * o
            blk.flux[0] = self.flux[0].data_ptr() + 8 * nv * o
            blk.flux[1] = self.flux[1].data_ptr() + 8 * nv * o
            blk.nx[:] = [B.nx[0], B.nx[1], 1]
            blk.dx[:] = [B.dx[0], B.dx[1], 1.0]
        self._blocks = blocks
        self.params = _params(cfg, exact)
        self.pack = ctypes.c_void_p()
        _capi.call("aph_pack_create", ctypes.byref(self.params), blocks, cfg.nblocks,
                   ctypes.byref(self.pack))
        self._table = amr_table(cfg)
        _capi.call("aph_pack_set_amr", self.pack, self._table, _bc_array(cfg))
        self._parts = None

    @property
    def block_packs(self):
        from . import _capi
        if self._parts is None:
            self._parts = []
            for b in range(self.cfg.nblocks):
                h = ctypes.c_void_p()
                _capi.call("aph_pack_partition", self.pack, b, 1, ctypes.byref(h))
                self._parts.append(h)
        return self._parts

    def close(self):
        from . import _capi
        lib = _capi.load()
        for h in self._parts or []:
            lib.aph_pack_destroy(h)
        self._parts = None
        if self.pack:
            lib.aph_pack_destroy(self.pack)
            self.pack = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class AmrDriver:
    """Per-kernel path on a refined pack: one launch per kernel per pack, or (per_block) one
    launch per kernel per meshblock; ghost fill and the flux correction are per pack."""

    def __init__(self, cfg: AmrConfig, cons0, exact=True, per_block=False):
        import torch
        from . import hydro
        self.cfg = cfg
        self.md = AmrMeshData(cfg, exact)
        self.md.cons.copy_(torch.as_tensor(np.ascontiguousarray(cons0)))
        self.per_block = per_block
        self.h = hydro
        self.time, self.ncycle = 0.0, 0
        self._fill()
        self._derived()
        self.dt = self._estimate()

    def _packs(self):
        return self.md.block_packs if self.per_block else [self.md.pack]

    def _fill(self):
        from . import _capi
        _capi.call("aph_hydro_fill_ghosts", self.md.pack, self.h.stream_handle())

    def _derived(self):
        for p in self._packs():
            self.h.ConsToPrim(self.md, pack=p)

    def _estimate(self):
        return min(self.h.EstimateTimestep(self.md, pack=p) for p in self._packs())

    def step(self, dt):
        cfg, md, h = self.cfg, self.md, self.h
        for s, (gam0, gam1, beta) in enumerate(h.STAGES[cfg.integrator]):
            if s == 0:
                md.u1.copy_(md.cons)
            recon = "dc" if (cfg.integrator == "vl2" and s == 0) else cfg.recon
            for p in self._packs():
                h.CalculateFluxes(md, recon, cfg.rsolver, pack=p)
            # the update reads the neighbours' fluxes (coarse-fine correction): all fluxes first
            for p in self._packs():
                h.UpdateWithFluxDivergence(md, gam0, gam1, beta * dt, pack=p)
                if cfg.gravity is not None:
                    h.ApplyGravity(md, cfg.gravity, beta * dt, pack=p)
            self._fill()
            self._derived()

    def run(self, nsteps=1 << 30, tlim=float("inf"), fixed_dt=0.0):
        taken = 0
        while taken < nsteps and self.time < tlim:
            dt = fixed_dt if fixed_dt > 0 else self.dt
            if fixed_dt <= 0 and (tlim - self.time) < dt:
                dt = tlim - self.time
            self.step(dt)
            self.time += dt
            self.ncycle += 1
            taken += 1
            self.dt = min(2.0 * dt, self._estimate())
        return taken

    def cons(self):
        import torch
        torch.cuda.synchronize()
        return self.md.cons.cpu().numpy()


class AmrStepper(_StepperBase):
    """Batched path on a refined pack: one persistent launch per stage over all blocks (the
    same aph_stepper_* handle as the uniform stepper, created with a face table)."""

    def __init__(self, cfg: AmrConfig, cons0, exact=True, tlim=None, fixed_dt=0.0):
        import torch
        from . import _capi
        from .hydro import require_cuda
        require_cuda()
        _capi.load()
        self.cfg = cfg
        self.exact = exact
        self.cons = torch.zeros(cfg.flat_size(), dtype=torch.float64, device="cuda")
        self.cons.copy_(torch.as_tensor(np.ascontiguousarray(cons0)))
        blocks = (_capi.aph_block * cfg.nblocks)()
        for b, B in enumerate(cfg.blocks):
            blocks[b].cons = self.cons.data_ptr() + 8 * cfg.nvar * cfg.offset[b]
            blocks[b].nx[:] = [B.nx[0], B.nx[1], 1]
            blocks[b].dx[:] = [B.dx[0], B.dx[1], 1.0]
        self._blocks = blocks
        self._table = amr_table(cfg)
        desc = _capi.aph_stepper_desc()
        desc.params = _params(cfg, exact)
        desc.integrator = _capi.INTEGRATOR[cfg.integrator]
        desc.nblocks = cfg.nblocks
        desc.blocks = ctypes.cast(blocks, ctypes.POINTER(_capi.aph_block))
        desc.nb[:] = [cfg.nblocks, 1, 1]
        desc.bc[:] = list(_bc_array(cfg))
        desc.use_gravity = 1 if cfg.gravity is not None else 0
        desc.gravity[:] = list(cfg.gravity) if cfg.gravity is not None else [0.0, 0.0, 0.0]
        desc.tlim = tlim if tlim is not None else 0.0
        desc.fixed_dt = fixed_dt
        desc.amr = ctypes.cast(self._table, ctypes.POINTER(_capi.aph_amr_block))
        self.h = ctypes.c_void_p()
        _capi.call("aph_stepper_create", ctypes.byref(desc), ctypes.byref(self.h))

    def interior_values(self):
        return self.cfg.nvar * self.cfg.zones()

    def tune_key(self):
        import torch
        cfg = self.cfg
        levels = ",".join("%d:%d" % kv for kv in sorted(cfg.level_counts().items()))
        return "%s|%s|amr|blocks%d|zones%d|levels%s|%s|%s|%s|exact%d" % (
            torch.cuda.get_device_name(), cfg.name, cfg.nblocks, cfg.zones(), levels, cfg.recon,
            cfg.rsolver, cfg.integrator, int(self.exact))


def with_tracers(cfg, cons5, nscalars=2):
    """(cfg, flat cons) of a refined problem with passive scalars (dyes) added: scalar k is
    rho * s_k, s_0 a band in y and s_1 a smooth pattern in x and y (as problems.with_tracers)."""
    import dataclasses
    tcfg = dataclasses.replace(cfg, nscalars=nscalars)
    cons = np.zeros(tcfg.flat_size())
    for b in range(tcfg.nblocks):
        src = cfg.block_view(cons5, b)
        dst = tcfg.block_view(cons, b)
        dst[:5] = src[:5]
        ng = tcfg.ng
        x, y = tcfg.cell_centers(b)
        rho = src[0, 0, ng:-ng, ng:-ng]
        dyes = [0.5 * (np.tanh((y - 0.25) / 0.05) - np.tanh((y - 0.75) / 0.05)),
                0.5 + 0.25 * np.sin(2 * math.pi * x) * np.cos(2 * math.pi * y)]
        for k in range(nscalars):
            dst[5 + k, 0, ng:-ng, ng:-ng] = rho * dyes[k % 2]
    return tcfg, cons


def uniform_as_amr(cfg):
    """The uniform 2D mesh `cfg` (mesh.MeshConfig) as an unrefined AmrConfig; block b and the
    flat layout match the uniform pack's (nblocks, nvar, 1, nj, ni) order."""
    assert cfg.ndim == 2 and cfg.block_nx[0] == cfg.block_nx[1]
    xmin, xmax = tuple(cfg.xmin[:2]), tuple(cfg.xmax[:2])
    bc = (tuple(cfg.bc[0]), tuple(cfg.bc[1]))
    leaves = build(tuple(cfg.mesh_nx[:2]), cfg.block_nx[0], cfg.block_nx[0], 0, xmin, xmax, bc,
                   lambda *a: False)
    return AmrConfig(leaves, cfg.ng, tuple(cfg.mesh_nx[:2]), xmin, xmax, bc, recon=cfg.recon,
                     rsolver=cfg.rsolver, integrator=cfg.integrator, gamma=cfg.gamma, cfl=cfg.cfl,
                     dfloor=cfg.dfloor, pfloor=cfg.pfloor, gravity=cfg.gravity,
                     name=cfg.name + "_as_amr", nscalars=cfg.nscalars)
