"""A rank's shard stepped by the oracle (test infrastructure): the engine interface of
apophis_gb300.shard.step over the oracle's single-block kernels, in the oracle mesh driver's
stage order (fluxes, update, gravity of each block; then the halo exchange and ConsToPrim of
the new state; the dt estimate after the last stage), so that ranks stepping their shards
with halo exchanges between stages must reproduce the single-process oracle run bit for bit.
"""
import numpy as np
import torch

from apophis_gb300 import shard
from apophis_gb300.hydro import STAGES
from oracle import oracle as O


class OracleShard:
    def __init__(self, cfg, parts, rank, cons_local, group=None):
        self.cfg = cfg
        self.plan = shard.plan_halo(cfg, parts, rank)
        self.group = group
        self.device = "cpu"
        self.u0 = torch.from_numpy(np.array(cons_local, dtype=np.float64, copy=True))
        shape = tuple(self.u0.shape)
        self.prim = np.zeros(shape)
        self.gamma = np.zeros(shape[:1] + (2,) + shape[2:])
        self.nstages = len(STAGES[cfg.integrator])
        self.time, self.ncycle = 0.0, 0
        shard.exchange(self.u0, self.plan, group)
        self._derive()
        self.dt = shard.global_dt(self.local_estimate(), group)

    def _derive(self):
        c, u = self.cfg, self.u0.numpy()
        for b in range(u.shape[0]):
            O.cons_to_prim(u[b], self.prim[b], self.gamma[b], c.block_nx, c.ng, c.ndim, c.gm1,
                           c.dfloor, c.pfloor)

    def stage(self, i):
        c, u = self.cfg, self.u0.numpy()
        if i == 0:
            self.u1 = u.copy()
        gam0, gam1, beta = STAGES[c.integrator][i]
        recon = "dc" if c.integrator == "vl2" and i == 0 else c.recon
        for b in range(u.shape[0]):
            flux = [np.zeros_like(u[b]) for _ in range(3)]
            O.calculate_fluxes(self.prim[b], self.gamma[b], flux, c.block_nx, c.ng, c.ndim, recon,
                               c.rsolver)
            O.update(u[b], self.u1[b], flux, c.block_nx, c.ng, c.ndim, c.dx, gam0, gam1,
                     beta * self.dt)
            if c.gravity is not None:
                O.apply_gravity(u[b], self.prim[b], c.block_nx, c.ng, c.ndim, c.gravity,
                                beta * self.dt)
        shard.exchange(self.u0, self.plan, self.group)
        self._derive()

    def local_estimate(self):
        c, u = self.cfg, self.u0.numpy()
        return min(O.estimate_dt(self.prim[b], u[b], c.block_nx, c.ng, c.ndim, c.dx, c.cfl, c.gm1)
                   for b in range(u.shape[0]))

    def end_step(self, estimate):
        self.time += self.dt
        self.ncycle += 1
        self.dt = min(2.0 * self.dt, estimate)
