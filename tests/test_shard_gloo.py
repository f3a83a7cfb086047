"""Sharded halo exchange and dt reduction with two CPU processes (gloo): every ghost cell a
rank fills equals the oracle's single-process ghost fill."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from apophis_gb300 import problems, shard
from apophis_gb300.mesh import MeshConfig


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _case(name):
    if name == "kh2d":
        return problems.kh2d(n=32, block=8, ng=2)
    if name == "rt2d":
        return problems.rt2d(nx=16, ny=48, block=(8, 8), ng=3)
    if name == "kh2d_tracers":  # passive scalars ride along in the exchange
        return problems.kh2d_tracers(n=32, block=8, ng=2)
    cfg = MeshConfig(ndim=3, mesh_nx=(16, 16, 16), block_nx=(8, 8, 8), ng=2,
                     bc=(("periodic", "periodic"), ("outflow", "reflecting"), ("reflecting", "outflow")),
                     recon="plm", rsolver="hlle")
    rng = np.random.Generator(np.random.PCG64(1))
    shape = cfg.pack_shape(5)
    rho = rng.uniform(0.5, 2.0, size=shape[:1] + shape[2:])
    v = rng.uniform(-0.5, 0.5, size=(shape[0], 3) + shape[2:])
    p = rng.uniform(0.5, 2.0, size=rho.shape)
    cons = np.empty(shape)
    cons[:, 0] = rho
    cons[:, 1:4] = rho[:, None] * v
    cons[:, 4] = p / cfg.gm1 + 0.5 * rho * (v ** 2).sum(axis=1)
    return cfg, cons


def _worker(rank, world, port, name, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        cfg, cons = _case(name)
        parts = shard.partition(cfg, world)
        plan = shard.plan_halo(cfg, parts, rank)
        local = torch.from_numpy(np.ascontiguousarray(cons[parts[rank]]))
        # poison the ghost cells: every one must be overwritten
        sk, sj, si = cfg.interior
        mask = torch.ones_like(local, dtype=torch.bool)
        mask[:, :, sk, sj, si] = False
        local[mask] = float("nan")
        shard.exchange(local, plan)
        dt = shard.global_dt(0.1 + rank)
        q.put((rank, parts[rank], local.numpy(), dt))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("name", ["kh2d", "rt2d", "box3d", "kh2d_tracers"])
def test_two_rank_exchange_matches_oracle(name):
    from oracle import oracle as O
    cfg, cons = _case(name)
    ref = O.Mesh(cfg)
    ref.set_cons(cons)          # the oracle fills every ghost cell (corners included)
    want = ref.get("cons")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, name, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    owned = set()
    for rank, blocks, local, dt in got:
        assert dt == 0.1
        owned |= set(blocks)
        assert np.array_equal(local, want[blocks]), (name, rank)
    assert owned == set(range(cfg.nblocks))


def _step_worker(rank, world, port, name, nsteps, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from shard_oracle import OracleShard
        cfg, cons = _case(name)
        parts = shard.partition(cfg, world)
        eng = OracleShard(cfg, parts, rank, cons[parts[rank]])
        shard.step(eng, nsteps)
        q.put((rank, parts[rank], eng.u0.numpy().copy(), eng.time, eng.dt, eng.ncycle))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("name", ["kh2d", "rt2d"])
def test_two_rank_sharded_steps_match_oracle(name):
    """Two ranks step their shards (halo exchange before every stage's reconstruction, dt
    reduced over the ranks) for 3 RK2 steps: the interiors, time and dt equal the single-
    process oracle run bit for bit (KH 2D periodic; RT with reflecting walls and gravity)."""
    from oracle import oracle as O
    nsteps = 3
    cfg, cons = _case(name)
    ref = O.Mesh(cfg)
    ref.set_cons(cons)
    ref.run(nsteps=nsteps)
    want, st = ref.get("cons"), ref.state()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_step_worker, args=(r, 2, port, name, nsteps, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    sk, sj, si = cfg.interior
    for rank, blocks, local, t, dt, ncycle in got:
        assert ncycle == nsteps and t == st["time"] and dt == st["dt"], (rank, t, dt)
        assert np.array_equal(local[:, :, sk, sj, si], want[blocks][:, :, sk, sj, si]), (name, rank)


def test_partition_is_balanced_and_contiguous_in_z_order():
    cfg, _ = problems.kh3d(n=64, block=16, ng=4)
    for nranks in (1, 2, 3, 4, 8):
        parts = shard.partition(cfg, nranks)
        sizes = [len(p) for p in parts]
        assert sum(sizes) == cfg.nblocks and max(sizes) - min(sizes) <= 1
        assert sorted(b for p in parts for b in p) == list(range(cfg.nblocks))
