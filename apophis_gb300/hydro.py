"""Host-side mirror of apophis's hydro package interface over the C ABI.

The names follow the reference: ``ConsToPrim`` (src/hydro/hydro.cpp:422-533),
``CalculateFluxes`` (hydro.cpp:535-744), ``EstimateTimestep`` (hydro.cpp:351-420),
Parthenon's ``UpdateWithFluxDivergence`` and the constant-g ``ApplyGravity``
(src/gravity/gravity.cpp:374-410), and ``Driver`` runs one RK step in the stage order
of ``ApophisDriver::MakeTaskCollection`` (src/apophis_driver.cpp:27-129).  PyTorch only
provides device memory and the current CUDA stream; all arithmetic runs in the CUDA
kernels of libaph_hydro.so.  There is no CPU fallback: without a CUDA device every
entry point raises.
"""
import ctypes

import numpy as np
import torch

from . import _capi
from .mesh import MeshConfig

# Low-storage RK coefficients (gam0, gam1, beta) per stage (Parthenon integrators).
STAGES = {
    "rk1": [(0.0, 1.0, 1.0)],
    "rk2": [(0.0, 1.0, 1.0), (0.5, 0.5, 0.5)],
    "rk3": [(0.0, 1.0, 1.0), (0.25, 0.75, 0.25), (2.0 / 3.0, 1.0 / 3.0, 2.0 / 3.0)],
    "vl2": [(0.0, 1.0, 0.5), (0.0, 1.0, 1.0)],
}


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("apophis_gb300 needs a CUDA device: the hydro path has no CPU "
                           "implementation")


def stream_handle(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def make_params(cfg: MeshConfig, exact=False, nvar=5):
    return _capi.aph_hydro_params(cfg.ndim, cfg.ng, nvar, _capi.RECON[cfg.recon],
                                  _capi.RSOLVER[cfg.rsolver], cfg.gm1, cfg.dfloor, cfg.pfloor,
                                  cfg.cfl, 1 if exact else 0)


class MeshData:
    """A pack of meshblocks resident in HBM (Parthenon ``MeshData<Real>``).

    Fields are torch tensors ``(nblocks, nvar, nk, nj, ni)``: ``cons``, ``prim``, ``u1``,
    ``flux[d]`` and ``gamma`` (2 components).  ``pack`` is the C-ABI handle over all
    blocks; ``block_packs`` (on demand) hold one handle per meshblock.

    face_fluxes: flux[d] shaped as Parthenon's face-centred arrays, one face longer along
    d (``(nblocks, nvar, nk, nj, ni + 1)`` along x1), passed to the library with their
    strides.  eos_lambda: also allocate the reference's ``eos_lambda`` field (3 components,
    zero-initialised), which ConsToPrim touches as the reference's does.
    """

    def __init__(self, cfg: MeshConfig, exact=True, device="cuda", face_fluxes=False,
                 eos_lambda=False):
        require_cuda()
        _capi.load()
        self.cfg = cfg
        self.exact = exact
        shape = cfg.pack_shape(cfg.nvar)
        kw = dict(dtype=torch.float64, device=device)
        self.cons = torch.zeros(shape, **kw)
        self.prim = torch.zeros(shape, **kw)
        self.u1 = torch.zeros(shape, **kw)
        self.gamma = torch.zeros(shape[:1] + (2,) + shape[2:], **kw)
        self.flux = []
        for d in range(3):
            if d >= cfg.ndim:
                self.flux.append(None)
                continue
            fshape = list(shape)
            if face_fluxes:
                fshape[4 - d] += 1  # one more face along d
            self.flux.append(torch.zeros(fshape, **kw))
        self.eos_lambda = (torch.zeros(shape[:1] + (3,) + shape[2:], **kw) if eos_lambda
                           else None)
        self.params = make_params(cfg, exact, cfg.nvar)
        self.pack = self._make_pack(range(cfg.nblocks))
        nb = (ctypes.c_int * 3)(*cfg.blocks_per_dim)
        bc = (ctypes.c_int * 6)(*[_capi.BC[cfg.bc[d][s]] for d in range(3) for s in range(2)])
        _capi.call("aph_pack_set_topology", self.pack, nb, bc)
        self._block_packs = None

    def _block_desc(self, b):
        cfg = self.cfg
        blk = _capi.aph_block()
        blk.cons = self.cons[b].data_ptr()
        blk.prim = self.prim[b].data_ptr()
        blk.gamma = self.gamma[b].data_ptr()
        blk.u1 = self.u1[b].data_ptr()
        for d in range(3):
            f = self.flux[d]
            blk.flux[d] = f[b].data_ptr() if f is not None else None
            if f is not None and tuple(f.shape) != tuple(self.cons.shape):
                blk.flux_stride[d][:] = [f.stride(1), f.stride(2), f.stride(3)]
            blk.nx[d] = cfg.block_nx[d]
            blk.dx[d] = cfg.dx[d]
        if self.eos_lambda is not None:
            blk.eos_lambda = self.eos_lambda[b].data_ptr()
        return blk

    def _make_pack(self, blocks):
        blocks = list(blocks)
        arr = (_capi.aph_block * len(blocks))(*[self._block_desc(b) for b in blocks])
        h = ctypes.c_void_p()
        _capi.call("aph_pack_create", ctypes.byref(self.params), arr, len(blocks), ctypes.byref(h))
        return h

    @property
    def block_packs(self):
        if self._block_packs is None:
            self._block_packs = [self._make_pack([b]) for b in range(self.cfg.nblocks)]
        return self._block_packs

    def close(self):
        lib = _capi.load()
        for h in ([self.pack] if getattr(self, "pack", None) else []) + (self._block_packs or []):
            lib.aph_pack_destroy(h)
        self.pack = None
        self._block_packs = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_cons(self, cons):
        self.cons.copy_(torch.as_tensor(np.ascontiguousarray(cons)).to(self.cons.device))


# ---- the reference's entry points ------------------------------------------------------
def ConsToPrim(md, pack=None, stream=None):
    _capi.call("aph_hydro_cons_to_prim", pack or md.pack, stream_handle(stream))


def CalculateFluxes(md, recon=None, rsolver=None, pack=None, stream=None):
    recon = _capi.RECON[recon or md.cfg.recon]
    rsolver = _capi.RSOLVER[rsolver or md.cfg.rsolver]
    _capi.call("aph_hydro_calculate_fluxes", pack or md.pack, recon, rsolver,
               stream_handle(stream))


def UpdateWithFluxDivergence(md, gam0, gam1, beta_dt, pack=None, stream=None):
    _capi.call("aph_hydro_update_with_flux_divergence", pack or md.pack, gam0, gam1, beta_dt,
               stream_handle(stream))


def EstimateTimestep(md, pack=None, stream=None):
    out = ctypes.c_double()
    _capi.call("aph_hydro_estimate_timestep", pack or md.pack, ctypes.byref(out),
               stream_handle(stream))
    return out.value


def ApplyGravity(md, g, beta_dt, pack=None, stream=None):
    ga = (ctypes.c_double * 3)(*g)
    _capi.call("aph_hydro_apply_gravity", pack or md.pack, ga, beta_dt, stream_handle(stream))


def History(md, pack=None, stream=None):
    """GlobalQuantHst (hydro.cpp:754-771): {"total_mass", "total_energy"} of the interiors."""
    out = (ctypes.c_double * 2)()
    _capi.call("aph_hydro_history", pack or md.pack, out, stream_handle(stream))
    return {"total_mass": out[0], "total_energy": out[1]}


def FillGhosts(md, stream=None):
    _capi.call("aph_hydro_fill_ghosts", md.pack, stream_handle(stream))


class Driver:
    """RK time stepping through the per-kernel entry points.

    ``per_block=False`` launches each kernel once per pack (the reference's Kokkos
    granularity); ``per_block=True`` launches each kernel once per meshblock (the plain
    per-meshblock path).  Stage order per src/apophis_driver.cpp:27-129: u1 <- u0 at
    stage 1, fluxes, flux-divergence update, gravity, boundary fill, FillDerived, and the
    dt estimate after the last stage.  dt policy: dt_n = min(2 dt_{n-1}, estimate),
    clipped at tlim.
    """

    def __init__(self, cfg: MeshConfig, cons0, exact=True, per_block=False):
        self.cfg = cfg
        self.md = MeshData(cfg, exact)
        self.per_block = per_block
        self.md.set_cons(cons0)
        self.time = 0.0
        self.ncycle = 0
        FillGhosts(self.md)
        self._derived()
        self.dt = self._estimate()

    def _packs(self):
        return self.md.block_packs if self.per_block else [self.md.pack]

    def _derived(self):
        for p in self._packs():
            ConsToPrim(self.md, pack=p)

    def _estimate(self):
        if not self.per_block:
            return EstimateTimestep(self.md)
        return min(EstimateTimestep(self.md, pack=p) for p in self._packs())

    def step(self, dt):
        cfg, md = self.cfg, self.md
        for s, (gam0, gam1, beta) in enumerate(STAGES[cfg.integrator]):
            if s == 0:
                md.u1.copy_(md.cons)
            recon = "dc" if (cfg.integrator == "vl2" and s == 0) else cfg.recon
            for p in self._packs():
                CalculateFluxes(md, recon, cfg.rsolver, pack=p)
                UpdateWithFluxDivergence(md, gam0, gam1, beta * dt, pack=p)
                if cfg.gravity is not None:
                    ApplyGravity(md, cfg.gravity, beta * dt, pack=p)
            FillGhosts(md)
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
        torch.cuda.synchronize()
        return self.md.cons.cpu().numpy()
