"""Host-side problem builders (CPU): the passive-scalar helpers, the floor-firing double
rarefaction and the ensemble's consistency checks, with the oracle as the checker."""
import numpy as np
import pytest

from apophis_gb300 import amr, ensemble, problems
from oracle import oracle as O


def _interior(cfg, a):
    sk, sj, si = cfg.interior
    return a[:, :, sk, sj, si]


def test_with_tracers_keeps_hydro_and_sets_dyes():
    cfg5, cons5 = problems.kh3d(n=16, block=8, ng=4)
    cfg, cons = problems.with_tracers(cfg5, cons5, nscalars=3)
    assert cfg.nvar == 8 and cons.shape == cfg.pack_shape(8)
    assert np.array_equal(cons[:, :5], cons5)
    rho = _interior(cfg, cons)[:, 0]
    for k in range(3):
        s = _interior(cfg, cons)[:, 5 + k] / rho
        assert np.all((s >= -1e-12) & (s <= 1.0 + 1e-12))  # concentrations in [0, 1]
    sk, sj, si = cfg.interior
    ghost = cons.copy()
    ghost[:, :, sk, sj, si] = 0.0
    assert not ghost[:, 5:].any()  # ghost cells are left to the drivers


def test_refined_tracers_match_block_layout():
    cfg5, cons5 = amr.small_test_mesh()
    cfg, cons = amr.with_tracers(cfg5, cons5, nscalars=2)
    assert cfg.nvar == 7 and cons.size == cfg.flat_size()
    for b in (0, cfg.nblocks // 2, cfg.nblocks - 1):
        assert np.array_equal(cfg.block_view(cons, b)[:5], cfg5.block_view(cons5, b))


def test_tracer_oracle_conserves_and_stays_bounded():
    cfg, cons = problems.kh2d_tracers(n=32, block=16, ng=2)
    m = O.Mesh(cfg)
    m.set_cons(cons)
    before = _interior(cfg, cons)[:, 5:].sum(axis=(0, 2, 3, 4))
    m.run(nsteps=10)
    out = _interior(cfg, m.get("cons"))
    assert np.allclose(out[:, 5:].sum(axis=(0, 2, 3, 4)), before, rtol=1e-13, atol=0)
    s = out[:, 5:] / out[:, :1]
    assert s.min() > -1e-3 and s.max() < 1.0 + 1e-3  # upwinded: no large over/undershoots


def test_double_rarefaction_fires_the_floor_in_some_blocks():
    cfg, cons = problems.rarefaction2d()
    m = O.Mesh(cfg)
    m.set_cons(cons)
    m.run(nsteps=4)
    u = _interior(cfg, m.get("cons"))
    ek = 0.5 * (u[:, 1] ** 2 + u[:, 2] ** 2 + u[:, 3] ** 2) / u[:, 0]
    p = cfg.gm1 * (u[:, 4] - ek)
    fired = [(p[b] < cfg.pfloor).any() for b in range(cfg.nblocks)]
    assert 0 < sum(fired) < cfg.nblocks  # a mix: floored blocks beside unfloored ones


def test_ensemble_members_must_share_scalars():
    a, _ = problems.blast2d(n=32, block=16, ng=4)
    b, _ = problems.with_tracers(*problems.blast2d(n=32, block=16, ng=4), nscalars=1)
    with pytest.raises(ValueError, match="nscalars"):
        ensemble.Ensemble([a, b], [0.1, 0.1])
    ens = ensemble.Ensemble([b, b], [0.1, 0.1])
    assert ens.nvar == 6
    flat = ens.pack([np.ones(b.pack_shape(6)), 2 * np.ones(b.pack_shape(6))])
    assert flat.size == 6 * ens.total_cells
    assert np.all(ens.unpack(flat, 1) == 2.0)
