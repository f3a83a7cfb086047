"""Adjoint of the hydro step (aph_adjoint_* in include/aph_hydro.h).

``Adjoint`` runs fixed-dt rollouts with step checkpointing and their reverse sweeps on
device tensors in pack layout (nblocks, 5, nk, nj, ni).  The torch.autograd wrapper lives
in the tests only.
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
        desc.params = make_params(cfg, exact=False)
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

    def forward(self, u0, dts, checkpoint_every=20):
        dts = [float(x) for x in dts]
        arr = (ctypes.c_double * len(dts))(*dts)
        out = self.empty()
        _capi.call("aph_adjoint_forward", self.h, _ptr(u0), len(dts), arr, int(checkpoint_every),
                   _ptr(out), stream_handle())
        return out

    def backward(self, lam_final):
        out = self.empty()
        _capi.call("aph_adjoint_backward", self.h, _ptr(lam_final), _ptr(out), stream_handle())
        return out
