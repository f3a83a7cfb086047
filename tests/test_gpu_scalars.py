"""Passive scalars (hydro/composition; fluxes upwinded by the mass flux, hydro.cpp:607-615)
on the per-kernel path and the batched stepper: every step bit-identical to the oracle in
exact mode, 1e-12 in fast mode, tracer mass conserved."""
import numpy as np
import pytest

from apophis_gb300 import hydro, problems
from apophis_gb300.stepper import Stepper
from oracle import oracle as O
from parity_util import assert_parity

pytestmark = pytest.mark.gpu

WORKLOADS = [
    ("kh2d_plm_hllc", lambda: problems.kh2d_tracers(n=48, block=16, ng=2)),
    ("kh2d_ppm_hlle", lambda: problems.kh2d_tracers(n=48, block=16, ng=3, recon="ppm", rsolver="hlle")),
    ("kh2d_dc_hlle", lambda: problems.kh2d_tracers(n=48, block=16, ng=2, recon="dc", rsolver="hlle")),
    ("kh3d_ppm_hllc", lambda: problems.with_tracers(*problems.kh3d(n=16, block=8, ng=4), nscalars=3)),
    ("sod_plm_lhllc", lambda: problems.with_tracers(*problems.sod(nx=128, rsolver="lhllc", block_nx=32), nscalars=1)),
]
IDS = [w[0] for w in WORKLOADS]


def _interior(cfg, a):
    sk, sj, si = cfg.interior
    return a[:, :, sk, sj, si]


@pytest.mark.parametrize("per_block", [False, True], ids=["per_pack", "per_block"])
@pytest.mark.parametrize("wl", WORKLOADS, ids=IDS)
def test_scalars_per_kernel_match_oracle(cuda, wl, per_block):
    cfg, cons = wl[1]()
    assert cfg.nvar > 5
    for exact in (True, False):
        nsteps = 3 if exact else 1
        m = O.Mesh(cfg)
        m.set_cons(cons)
        m.run(nsteps=nsteps)
        d = hydro.Driver(cfg, cons, exact=exact, per_block=per_block)
        d.run(nsteps=nsteps)
        if exact:
            assert d.time == m.state()["time"]
        assert_parity(_interior(cfg, d.cons()), _interior(cfg, m.get("cons")), exact, what="cons")
        d.md.close()


@pytest.mark.parametrize("exact", [True, False], ids=["exact", "fast"])
@pytest.mark.parametrize("wl", WORKLOADS, ids=IDS)
def test_scalars_stepper_match_oracle(cuda, wl, exact):
    cfg, cons = wl[1]()
    m = O.Mesh(cfg)
    m.set_cons(cons)
    st = Stepper(cfg, cons, exact=exact)
    for _ in range(3 if exact else 1):
        m.run(nsteps=1)
        st.step(1)
        if exact:
            assert st.status()["dt"] == m.state()["dt"]
        assert_parity(_interior(cfg, st.state()), _interior(cfg, m.get("cons")), exact, what="cons")
    st.close()


@pytest.mark.parametrize("make,lines", [
    (lambda: problems.with_tracers(*problems.kh3d(n=16, block=8, ng=4), nscalars=2), [6, 6, 6]),
    (lambda: problems.kh2d_tracers(n=64, block=32, ng=4, recon="ppm", rsolver="hllc"), [6, 6, 0]),
])
def test_scalars_tma_windows_match_plain_loads(cuda, make, lines):
    """TMA windows carrying nvar > 5 variables: bit-identical to plain loads (interiors: ghost
    cells hold stage inputs, which plain-load launches read at their sources)."""
    cfg, cons = make()
    outs = []
    for tma in (0, 1):
        st = Stepper(cfg, cons, exact=False)
        c = st.config
        c.update(lines=lines, tma=tma, schedule=2)
        st.set_config(c)
        st.step(3)
        outs.append((_interior(cfg, st.state()), st.status()))
        st.close()
    assert np.array_equal(outs[1][0], outs[0][0]) and outs[1][1] == outs[0][1]


def test_scalars_stepper_autotune_and_conservation(cuda):
    cfg, cons = problems.with_tracers(*problems.kh3d(n=32, block=16, ng=4), nscalars=2)
    st = Stepper(cfg, cons, exact=False)
    st.autotune(trial_steps=2)
    st.step(10)
    out = _interior(cfg, st.state())
    for k in range(cfg.nscalars):
        before = _interior(cfg, cons)[:, 5 + k].sum()
        assert abs(out[:, 5 + k].sum() - before) <= 1e-12 * abs(before)
    st.close()


def test_tracer_mass_conserved(cuda):
    cfg, cons = problems.kh2d_tracers(n=64, block=32, ng=2)
    d = hydro.Driver(cfg, cons, exact=False)
    d.run(nsteps=20)
    out = _interior(cfg, d.cons())
    for k in range(cfg.nscalars):
        before = _interior(cfg, cons)[:, 5 + k].sum()
        assert abs(out[:, 5 + k].sum() - before) <= 1e-12 * abs(before)
    d.md.close()


def test_scalars_rejected_where_not_carried(cuda):
    from apophis_gb300 import adjoint
    cfg, cons = problems.kh2d_tracers(n=32, block=16, ng=2)
    with pytest.raises(Exception, match="passive scalars"):
        adjoint.Adjoint(cfg)


def _amr_interiors(cfg, flat):
    ng = cfg.ng
    return np.concatenate([cfg.block_view(flat, b)[:, 0, ng:-ng, ng:-ng].reshape(cfg.nvar, -1)
                           for b in range(cfg.nblocks)], axis=1)


@pytest.mark.parametrize("path", ["pack", "block", "stepper"])
def test_scalars_refined_mesh_exact(cuda, path):
    """Passive scalars on the two-level mesh: ghost map (copy, restriction, prolongation) and
    coarse-fine flux correction of the scalars, bit-identical to the refined-mesh oracle."""
    from apophis_gb300 import amr
    cfg, cons = amr.with_tracers(*amr.small_test_mesh(), nscalars=2)
    m = O.AmrMesh(cfg)
    m.set_cons(cons)
    m.run(nsteps=4)
    if path == "stepper":
        s = amr.AmrStepper(cfg, cons, exact=True)
        s.step(4)
        assert s.status()["time"] == m.state()["time"]
        got = s.state()
        s.close()
    else:
        d = amr.AmrDriver(cfg, cons, exact=True, per_block=(path == "block"))
        d.run(nsteps=4)
        assert d.time == m.state()["time"]
        got = d.cons()
        d.md.close()
    assert np.array_equal(_amr_interiors(cfg, got), _amr_interiors(cfg, m.get()))


def test_scalars_refined_mesh_fast_and_conserved(cuda):
    from apophis_gb300 import amr
    cfg, cons = amr.with_tracers(*amr.small_test_mesh(), nscalars=2)
    m = O.AmrMesh(cfg)
    m.set_cons(cons)
    m.run(nsteps=1)
    s = amr.AmrStepper(cfg, cons, exact=False)
    s.step(1)
    g, w = _amr_interiors(cfg, s.state()), _amr_interiors(cfg, m.get())
    for v in range(cfg.nvar):
        scale = np.abs(w[1:4]).max() if 1 <= v <= 3 else np.abs(w[v]).max()
        assert np.abs(g[v] - w[v]).max() <= 1e-12 * scale, v
    vol = np.concatenate([np.full(B.nx[0] * B.nx[1], B.dx[0] * B.dx[1]) for B in cfg.blocks])
    before = (_amr_interiors(cfg, cons)[5:] * vol).sum(axis=1)
    s.step(20)
    after = (_amr_interiors(cfg, s.state())[5:] * vol).sum(axis=1)
    assert np.all(np.abs(after - before) <= 1e-12 * np.abs(before))
    s.close()


def test_scalars_ensemble_members_match_oracle(cuda):
    """An ensemble whose members carry passive scalars: every member bit-identical (exact) to
    the oracle run of that member alone."""
    from apophis_gb300 import ensemble
    rng = np.random.Generator(np.random.PCG64(5))
    cfgs, conses = [], []
    for n in (32, 48, 32):
        cfg, cons = problems.with_tracers(*problems.blast2d(
            n=n, block=16, ng=4, r0=float(rng.uniform(0.1, 0.3)),
            gamma=float(rng.uniform(1.4, 5.0 / 3.0))), nscalars=2)
        cfgs.append(cfg)
        conses.append(cons)
    ens = ensemble.Ensemble(cfgs, [0.05] * len(cfgs))
    st = ensemble.EnsembleStepper(ens, ens.pack(conses), exact=True)
    st.step(4)
    got = st.state()
    for m, cfg in enumerate(cfgs):
        o = O.Mesh(cfg)
        o.set_cons(conses[m])
        o.run(nsteps=4)
        assert np.array_equal(_interior(cfg, ens.unpack(got, m)), _interior(cfg, o.get())), m
    st.close()
    from apophis_gb300 import adjoint
    with pytest.raises(Exception, match="passive scalars"):
        adjoint.EnsembleAdjoint(ens)


def test_scalars_with_floors_exact(cuda):
    """Passive scalars where the pressure floor fires: the stepper and the per-kernel path stay
    bit-identical to the oracle (scalar concentrations use the floored density)."""
    cfg, cons = problems.with_tracers(*problems.rarefaction2d(), nscalars=2)
    m = O.Mesh(cfg)
    m.set_cons(cons)
    st = Stepper(cfg, cons, exact=True)
    d = hydro.Driver(cfg, cons, exact=True)
    for _ in range(6):
        m.run(nsteps=1)
        st.step(1)
        d.run(nsteps=1)
        want = _interior(cfg, m.get("cons"))
        assert np.array_equal(_interior(cfg, st.state()), want)
        assert np.array_equal(_interior(cfg, d.cons()), want)
    st.close()
    d.md.close()


def test_scalars_ensemble_tma_matches_plain_loads(cuda):
    """An ensemble of equal blocks carrying scalars: TMA windows over 7 variables give the same
    bits as plain loads."""
    from apophis_gb300 import ensemble
    cfgs, conses = [], []
    for r0 in (0.1, 0.2):
        cfg, cons = problems.with_tracers(*problems.blast2d(n=32, block=16, ng=4, r0=r0), nscalars=2)
        cfgs.append(cfg)
        conses.append(cons)
    ens = ensemble.Ensemble(cfgs, [0.05, 0.05])
    outs = []
    for tma in (0, 1):
        st = ensemble.EnsembleStepper(ens, ens.pack(conses), exact=False)
        c = st.config
        c.update(lines=[4, 4, 0], tma=tma)
        st.set_config(c)
        st.step(3)
        outs.append(st.state())
        st.close()
    for m, cfg in enumerate(ens.members):  # interiors (ghost cells hold stage inputs)
        assert np.array_equal(_interior(cfg, ens.unpack(outs[0], m)), _interior(cfg, ens.unpack(outs[1], m))), m


def test_scalars_interiors_round_trip(cuda):
    import torch
    cfg, cons = problems.with_tracers(*problems.kh3d(n=16, block=8, ng=4), nscalars=2)
    st = Stepper(cfg, cons, exact=True)
    st.step(1)
    buf = torch.empty(st.interior_shape(), dtype=torch.float64, pin_memory=True)
    assert buf.shape[1] == 7
    st.store_interiors(buf)
    torch.cuda.synchronize()
    assert np.array_equal(buf.numpy(), _interior(cfg, st.state()))
    st.close()
