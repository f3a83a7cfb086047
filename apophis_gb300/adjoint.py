"""Adjoint of the hydro step (aph_adjoint_* in include/aph_hydro.h).

``Adjoint`` runs fixed-dt rollouts with step checkpointing and their reverse sweeps on
device tensors in pack layout (nblocks, 5, nk, nj, ni); ``EnsembleAdjoint`` does the same
for an ensemble (every member's reverse sweep in the same launches, a dt per member and
step).  The torch.autograd wrapper lives in the tests only.
"""
import ctypes

import torch

from . import _capi
from .hydro import make_params, require_cuda, stream_handle
from .mesh import MeshConfig


def _ptr(t):
    assert t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()
    return ctypes.c_void_p(t.data_ptr())


class Adjoint:
    def __init__(self, cfg: MeshConfig):
        require_cuda()
        _capi.load()
        self.cfg = cfg
        blocks = (_capi.aph_block * cfg.nblocks)()
        for b in range(cfg.nblocks):
            for d in range(3):
                blocks[b].nx[d] = cfg.block_nx[d]
                blocks[b].dx[d] = cfg.dx[d]
            blocks[b].cons = 1  # unused by the adjoint, must be non-null
        self._blocks = blocks
        desc = _capi.aph_stepper_desc()
        desc.params = make_params(cfg, exact=False, nvar=cfg.nvar)
        desc.integrator = _capi.INTEGRATOR[cfg.integrator]
        desc.nblocks = cfg.nblocks
        desc.blocks = ctypes.cast(blocks, ctypes.POINTER(_capi.aph_block))
        desc.nb[:] = list(cfg.blocks_per_dim)
        desc.bc[:] = [_capi.BC[cfg.bc[d][s]] for d in range(3) for s in range(2)]
        self.h = ctypes.c_void_p()
        _capi.call("aph_adjoint_create", ctypes.byref(desc), ctypes.byref(self.h))
        self.shape = cfg.pack_shape(5)

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            _capi.load().aph_adjoint_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def empty(self):
        return torch.zeros(self.shape, dtype=torch.float64, device="cuda")

    def step(self, u, dt):
        out = self.empty()
        _capi.call("aph_adjoint_step", self.h, _ptr(u), float(dt), _ptr(out), stream_handle())
        return out

    def step_vjp(self, u, dt, lam_next):
        out = self.empty()
        _capi.call("aph_adjoint_step_vjp", self.h, _ptr(u), float(dt), _ptr(lam_next), _ptr(out),
                   stream_handle())
        return out

    def autotune(self, u):
        """Tune the forward stepper's launch configuration on the state u."""
        _capi.call("aph_adjoint_autotune", self.h, _ptr(u), stream_handle())

    def forward(self, u0, dts, checkpoint_every=20):
        dts = [float(x) for x in dts]
        arr = (ctypes.c_double * len(dts))(*dts)
        out = self.empty()
        _capi.call("aph_adjoint_forward", self.h, _ptr(u0), len(dts), arr, int(checkpoint_every),
                   _ptr(out), stream_handle())
        return out

    def forward_members(self, u0, dts, checkpoint_every=20):
        """dts: nsteps rows of one dt per member."""
        rows = [[float(x) for x in r] for r in dts]
        flat = [x for r in rows for x in r]
        arr = (ctypes.c_double * len(flat))(*flat)
        out = self.empty()
        _capi.call("aph_adjoint_forward_members", self.h, _ptr(u0), len(rows), arr,
                   int(checkpoint_every), _ptr(out), stream_handle())
        return out

    def backward(self, lam_final):
        out = self.empty()
        _capi.call("aph_adjoint_backward", self.h, _ptr(lam_final), _ptr(out), stream_handle())
        return out


class EnsembleAdjoint(Adjoint):
    """Adjoint of an ensemble's step (apophis_gb300.ensemble.Ensemble): the state is the flat
    pack of all members (blocks of equal size); members keep their own gamma and dt."""

    def __init__(self, ens):
        from .ensemble import EnsembleStepper
        require_cuda()
        _capi.load()
        self.ens = ens
        c0 = ens.members[0]
        nb = ens.nblocks
        blks = ens.blocks()
        for B in blks:
            if B.nx != blks[0].nx:
                raise ValueError("the adjoint needs ensemble blocks of equal size")
        blocks = (_capi.aph_block * nb)()
        for b, B in enumerate(blks):
            blocks[b].cons = 1  # unused by the adjoint, must be non-null
            blocks[b].nx[:] = [B.nx[0], B.nx[1], 1]
            blocks[b].dx[:] = [B.dx[0], B.dx[1], 1.0]
        table = EnsembleStepper.face_table(blks)
        self._member = (ctypes.c_int * nb)(*ens.member_of)
        self._gm1 = (ctypes.c_double * ens.nmembers)(*[c.gm1 for c in ens.members])
        self._ens = _capi.aph_ensemble(ens.nmembers, self._member, self._gm1, None)
        self._blocks, self._table = blocks, table
        desc = _capi.aph_stepper_desc()
        desc.params = _capi.aph_hydro_params(2, c0.ng, ens.nvar, _capi.RECON[c0.recon],
                                             _capi.RSOLVER[c0.rsolver], c0.gm1, c0.dfloor,
                                             c0.pfloor, c0.cfl, 0)
        desc.integrator = _capi.INTEGRATOR[c0.integrator]
        desc.nblocks = nb
        desc.blocks = ctypes.cast(blocks, ctypes.POINTER(_capi.aph_block))
        desc.nb[:] = [nb, 1, 1]
        desc.bc[:] = [_capi.BC[c0.bc[d][s]] for d in range(2) for s in range(2)] + [0, 0]
        desc.amr = ctypes.cast(table, ctypes.POINTER(_capi.aph_amr_block))
        desc.ensemble = ctypes.pointer(self._ens)
        self.h = ctypes.c_void_p()
        _capi.call("aph_adjoint_create", ctypes.byref(desc), ctypes.byref(self.h))
        self.shape = (5 * ens.total_cells,)
