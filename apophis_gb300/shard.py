"""Sharding a uniform block grid over ranks (one GPU per rank): block partition, halo
exchange of the ghost zones between ranks, the dt min-reduction, and the sharded RK step that
strings them together -- the exchange steps of the reference's MPI driver
(apophis_driver.cpp:68-104 boundary communication, and the global dt min of EstimateTimestep).

``step(engine)`` runs one RK step of a rank's shard: every stage exchanges the halo and
advances the shard's blocks, then the ranks' dt estimates are reduced to their minimum and
the dt policy applied.  ``GpuShard`` is the engine of the CUDA path: the batched stepper over
the rank's blocks, driven stage by stage with the ghost cells the exchange filled
(aph_stepper_stage with APH_STAGE_GHOSTS_GIVEN, aph_stepper_local_dt, aph_stepper_end_step).

The partition gives each rank a contiguous range of blocks in Z (Morton) order.  The exchange
is planned from global metadata only (every rank derives the same plan): every ghost cell of
a local block has a source cell (global index mapping with the physical boundaries, as the
ghost fill does), and ghosts whose source lives on another rank are gathered there, sent in
one message per peer, and scattered into the ghost cells (with the reflecting sign flip).
Data stay on the ranks' devices; torch.distributed moves them (NCCL between GPUs, gloo on
CPU), with no host round trip on the GPU path.
"""
import dataclasses
import ctypes
from dataclasses import dataclass
from typing import Dict, List

import numpy as np
import torch
import torch.distributed as dist

from .mesh import IM1, IM2, IM3, MeshConfig

BC_PERIODIC, BC_OUTFLOW, BC_REFLECT = "periodic", "outflow", "reflecting"


def _morton(i, j, k):
    code = 0
    for bit in range(21):
        code |= ((i >> bit) & 1) << (3 * bit) | ((j >> bit) & 1) << (3 * bit + 1) | ((k >> bit) & 1) << (3 * bit + 2)
    return code


def partition(cfg: MeshConfig, nranks: int) -> List[List[int]]:
    """Blocks of each rank: contiguous ranges of the Z-order curve, sizes differing by <= 1."""
    nb = cfg.blocks_per_dim
    blocks = sorted(range(cfg.nblocks),
                    key=lambda b: _morton(b % nb[0], (b // nb[0]) % nb[1], b // (nb[0] * nb[1])))
    out, start = [], 0
    for r in range(nranks):
        n = cfg.nblocks // nranks + (1 if r < cfg.nblocks % nranks else 0)
        out.append(sorted(blocks[start:start + n]))
        start += n
    return out


def _map(g, n, lo, hi):
    """Global index g (possibly outside 0..n-1) -> (source index, mirrored)."""
    if g < 0:
        if lo == BC_PERIODIC:
            return g + n, False
        if lo == BC_OUTFLOW:
            return 0, False
        return -1 - g, True
    if g >= n:
        if hi == BC_PERIODIC:
            return g - n, False
        if hi == BC_OUTFLOW:
            return n - 1, False
        return 2 * n - 1 - g, True
    return g, False


@dataclass
class HaloPlan:
    """Ghost-cell sources of one rank's blocks, grouped by the rank that owns them."""
    rank: int
    owned: List[int]
    # per peer: flat indices (into this rank's stacked local blocks) of the values to send
    send: Dict[int, np.ndarray]
    # per peer: flat destination indices of the received values, and their sign (+1 / -1)
    recv: Dict[int, np.ndarray]
    recv_sign: Dict[int, np.ndarray]
    _dev: Dict = dataclasses.field(default_factory=dict, repr=False)

    def on(self, device, dtype):
        """The plan's index and sign arrays as tensors on device, made once per device."""
        key = (str(device), dtype)
        if key not in self._dev:
            self._dev[key] = (
                {q: torch.as_tensor(v, device=device) for q, v in self.send.items()},
                {q: torch.as_tensor(v, device=device) for q, v in self.recv.items()},
                {q: torch.as_tensor(v, dtype=dtype, device=device) for q, v in self.recv_sign.items()})
        return self._dev[key]


def plan_halo(cfg: MeshConfig, parts: List[List[int]], rank: int, nvar: int = None) -> HaloPlan:
    nvar = cfg.nvar if nvar is None else nvar  # 5 hydro variables, then the passive scalars
    ng, nd = cfg.ng, cfg.ndim
    bn = cfg.block_nx
    nb = cfg.blocks_per_dim
    N = [bn[d] * nb[d] for d in range(3)]
    shape = cfg.pack_shape(nvar)[1:]  # (nvar, nk, nj, ni)
    ncell = int(np.prod(shape[1:]))
    owner = {b: r for r, bl in enumerate(parts) for b in bl}
    slot = [{b: s for s, b in enumerate(bl)} for bl in parts]
    start = [ng if d < nd else 0 for d in range(3)]
    ext = [bn[d] + 2 * ng if d < nd else 1 for d in range(3)]

    def block_plan(b):
        """(dst cell, src block, src cell, flip per dim) for every ghost cell of block b."""
        loc = (b % nb[0], (b // nb[0]) % nb[1], b // (nb[0] * nb[1]))
        out = []
        for k in range(ext[2]):
            for j in range(ext[1]):
                for i in range(ext[0]):
                    e = (i, j, k)
                    ghost = any(d < nd and (e[d] < ng or e[d] >= ng + bn[d]) for d in range(3))
                    if not ghost:
                        continue
                    src, flips = [0, 0, 0], [False, False, False]
                    for d in range(3):
                        if d >= nd:
                            continue
                        g = loc[d] * bn[d] + e[d] - ng
                        src[d], flips[d] = _map(g, N[d], cfg.bc[d][0], cfg.bc[d][1])
                    sb = [src[d] // bn[d] if d < nd else 0 for d in range(3)]
                    sblk = (sb[2] * nb[1] + sb[1]) * nb[0] + sb[0]
                    sc = [src[d] - sb[d] * bn[d] + start[d] for d in range(3)]
                    out.append(((k * ext[1] + j) * ext[0] + i, sblk,
                                (sc[2] * ext[1] + sc[1]) * ext[0] + sc[0], tuple(flips)))
        return out

    # what every rank receives, grouped by sender (computed for all ranks: the plan is global)
    recv_lists = [dict() for _ in parts]
    for r, bl in enumerate(parts):
        for b in bl:
            for dst, sblk, scell, flips in block_plan(b):
                q = owner[sblk]
                lst = recv_lists[r].setdefault(q, [])
                for v in range(nvar):
                    sign = -1.0 if (v == IM1 and flips[0]) or (v == IM2 and flips[1]) or \
                        (v == IM3 and flips[2]) else 1.0
                    lst.append((slot[r][b] * nvar * ncell + v * ncell + dst,
                                slot[q][sblk] * nvar * ncell + v * ncell + scell, sign))
    send, recv, recv_sign = {}, {}, {}
    for q, lst in recv_lists[rank].items():
        recv[q] = np.array([x[0] for x in lst], dtype=np.int64)
        recv_sign[q] = np.array([x[2] for x in lst])
    for r in range(len(parts)):
        if rank in recv_lists[r]:
            send[r] = np.array([x[1] for x in recv_lists[r][rank]], dtype=np.int64)
    return HaloPlan(rank, parts[rank], send, recv, recv_sign)


def exchange(local: torch.Tensor, plan: HaloPlan, group=None):
    """Fill the ghost cells of this rank's blocks, local (len(owned), nvar, nk, nj, ni), in place.
    Values whose source block is local are copied directly; the others travel one message per
    peer (point-to-point, all posted before any wait)."""
    flat = local.view(-1)
    dev = local.device
    send_idx, recv_idx, recv_sign = plan.on(dev, local.dtype)
    bufs = {q: flat.index_select(0, i) for q, i in send_idx.items()}
    me = plan.rank
    incoming = {q: torch.empty(len(v), dtype=local.dtype, device=dev) for q, v in plan.recv.items()
                if q != me}
    ops = []
    for q, buf in bufs.items():
        if q != me:
            ops.append(dist.P2POp(dist.isend, buf, q, group))
    for q, buf in incoming.items():
        ops.append(dist.P2POp(dist.irecv, buf, q, group))
    reqs = dist.batch_isend_irecv(ops) if ops else []
    if me in plan.recv:  # sources on this rank
        flat.index_copy_(0, recv_idx[me], bufs[me] * recv_sign[me])
    for r in reqs:
        r.wait()
    for q, buf in incoming.items():
        flat.index_copy_(0, recv_idx[q], buf * recv_sign[q])


def global_dt(local_dt: float, group=None, device="cpu") -> float:
    """The step's dt: the minimum of every rank's estimate (an allreduce-min; the estimate
    itself without a process group)."""
    if not (dist.is_available() and dist.is_initialized()):
        return float(local_dt)
    t = torch.tensor([local_dt], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MIN, group=group)
    return float(t.item())


def step(engine, nsteps=1, group=None):
    """nsteps sharded RK steps of one rank's engine.  The engine provides ``nstages``,
    ``stage(i)`` (exchange the halo, then advance stage i of the step), ``local_estimate()``
    (cfl * min over its interior cells of the new state) and ``end_step(estimate)`` (the dt
    policy with the estimate of all ranks); ``device`` is where the dt reduction runs."""
    for _ in range(nsteps):
        for i in range(engine.nstages):
            engine.stage(i)
        est = global_dt(engine.local_estimate(), group, engine.device)
        engine.end_step(est)


@dataclass
class _ShardConfig:
    """A rank's blocks as a pack of their own: nlocal blocks in a row, with the mesh's dx."""
    base: MeshConfig
    nlocal: int

    def mesh(self) -> MeshConfig:
        b = self.base
        bn = b.block_nx
        # the cell widths of the blocks are passed explicitly (the mesh's, bit for bit); the
        # boundaries of the local pack never act (the exchange fills every ghost cell)
        return dataclasses.replace(b, mesh_nx=(bn[0] * self.nlocal, bn[1], bn[2]),
                                   bc=(("periodic", "periodic"),) * 3)


class GpuShard:
    """A rank's blocks on its GPU, stepped by the batched stepper stage by stage, with the
    ghost cells filled by the halo exchange before each stage."""

    def __init__(self, cfg: MeshConfig, parts: List[List[int]], rank: int, cons_local,
                 exact=True, tlim=None, group=None):
        from . import _capi
        from .hydro import STAGES, stream_handle
        from .stepper import Stepper
        self._capi, self._stream = _capi, stream_handle
        self.cfg = cfg
        self.plan = plan_halo(cfg, parts, rank)
        self.group = group
        local_cfg = _ShardConfig(cfg, len(parts[rank])).mesh()
        self.st = Stepper(local_cfg, cons_local, exact=exact, tlim=tlim, dx=cfg.dx)
        # the stepper's dt_0 is this rank's estimate: reduce it over the ranks
        self.device = self.st.cons.device
        s = self.st.status()
        dt0 = global_dt(s["dt"], group, self.device)
        _capi.call("aph_stepper_set_clock", self.st.h, s["time"], dt0, s["ncycle"], stream_handle())
        self.nstages = len(STAGES[cfg.integrator])

    @property
    def cons(self):
        return self.st.cons

    def stage(self, i):
        exchange(self.st.cons, self.plan, self.group)
        self._capi.call("aph_stepper_stage", self.st.h, i, self._capi.APH_STAGE_GHOSTS_GIVEN,
                        self._stream())

    def local_estimate(self):
        out = ctypes.c_double()
        self._capi.call("aph_stepper_local_dt", self.st.h, ctypes.byref(out), self._stream())
        return out.value

    def end_step(self, estimate):
        self._capi.call("aph_stepper_end_step", self.st.h, float(estimate), self._stream())

    def status(self):
        return self.st.status()

    def close(self):
        self.st.close()
