"""Ensembles: independent blast problems with their own gamma, dt and clock batched in one
stepper; every member against the oracle run of that member alone."""
import numpy as np
import pytest

from apophis_gb300 import ensemble, problems
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def small_ensemble(recon="ppm", rsolver="hllc", integrator="rk2", tlim=0.02, seed=3):
    rng = np.random.Generator(np.random.PCG64(seed))
    cfgs, conses = [], []
    for m, n in enumerate((32, 48, 64, 32, 48)):
        cfg, cons = problems.blast2d(n=n, block=16, ng=4 if recon == "ppm" else 2,
                                     r0=float(rng.uniform(0.1, 0.3)),
                                     gamma=float(rng.uniform(1.4, 5.0 / 3.0)), recon=recon,
                                     rsolver=rsolver, integrator=integrator)
        cfgs.append(cfg)
        conses.append(cons)
    tl = [tlim * (1.0 + 0.25 * m) for m in range(len(cfgs))]  # members end at different times
    ens = ensemble.Ensemble(cfgs, tl)
    return ens, conses, ens.pack(conses)


def _interior(cfg, a):
    sk, sj, si = cfg.interior
    return a[:, :, sk, sj, si]


@pytest.mark.parametrize("recon,rsolver,integrator", [("ppm", "hllc", "rk2"), ("plm", "hlle", "rk3")])
def test_members_match_oracle_exact(cuda, recon, rsolver, integrator):
    ens, conses, flat = small_ensemble(recon, rsolver, integrator)
    st = ensemble.EnsembleStepper(ens, flat, exact=True)
    st.step(5)
    ms = st.member_status()
    got = st.state()
    for m, cfg in enumerate(ens.members):
        o = O.Mesh(cfg)
        o.set_cons(conses[m])
        o.run(nsteps=5, tlim=ens.tlim[m])
        s = o.state()
        assert ms["ncycle"][m] == s["ncycle"] and ms["time"][m] == s["time"] and ms["dt"][m] == s["dt"]
        assert np.array_equal(_interior(cfg, ens.unpack(got, m)), _interior(cfg, o.get())), m
    st.close()


def test_members_run_to_their_end_times(cuda):
    ens, conses, flat = small_ensemble(tlim=0.01)
    st = ensemble.EnsembleStepper(ens, flat, exact=True)
    st.run_to_end(chunk=4)
    ms = st.member_status()
    got = st.state()
    for m, cfg in enumerate(ens.members):
        assert ms["time"][m] == pytest.approx(ens.tlim[m], rel=0, abs=1e-15) and ms["dt"][m] == 0.0
        o = O.Mesh(cfg)
        o.set_cons(conses[m])
        o.run(tlim=ens.tlim[m])
        assert o.state()["ncycle"] == ms["ncycle"][m]
        assert np.array_equal(_interior(cfg, ens.unpack(got, m)), _interior(cfg, o.get())), m
    assert st.status()["dt"] == 0.0
    st.close()


def test_members_fast_one_step(cuda):
    ens, conses, flat = small_ensemble()
    st = ensemble.EnsembleStepper(ens, flat, exact=False)
    st.step(1)
    got = st.state()
    for m, cfg in enumerate(ens.members):
        o = O.Mesh(cfg)
        o.set_cons(conses[m])
        o.run(nsteps=1)
        g, w = _interior(cfg, ens.unpack(got, m)), _interior(cfg, o.get())
        mom = np.abs(w[:, 1:4]).max()
        for v in range(5):
            scale = mom if 1 <= v <= 3 else np.abs(w[:, v]).max()
            assert np.abs(g[:, v] - w[:, v]).max() <= 1e-12 * scale, (m, v)
    st.close()


def test_ensemble_configs_agree(cuda):
    ens, conses, flat = small_ensemble()
    ref = None
    for sched in (0, 1, 2):
        st = ensemble.EnsembleStepper(ens, flat, exact=True)
        c = dict(st.config, schedule=sched)
        st.set_config(c)
        st.step(3)
        out = st.state()
        st.close()
        if ref is None:
            ref = out
        else:
            assert np.array_equal(out, ref)


def test_blast_ensemble_workload_runs(cuda):
    ens, flat = ensemble.blast_ensemble()
    assert ens.nmembers == 64 and ens.nblocks == 1814
    st = ensemble.EnsembleStepper(ens, flat, exact=False)
    st.step(2)
    ms = st.member_status()
    assert all(c == 2 for c in ms["ncycle"]) and all(d > 0 for d in ms["dt"])
    # mass of every member is conserved (periodic boxes)
    got = st.state()
    for m, cfg in enumerate(ens.members):
        a, b = ens.unpack(got, m), ens.unpack(flat, m)
        assert abs(_interior(cfg, a)[:, 0].sum() - _interior(cfg, b)[:, 0].sum()) <= 1e-12 * _interior(cfg, b)[:, 0].sum()
    st.close()


def _adjoint_ensemble(seed=5, recon="ppm"):
    """Three members of 16^2 blocks (32^2, 48^2, 64^2 grids), HLLC, smooth KH data, each with
    its own gamma."""
    from apophis_gb300 import problems as P
    rng = np.random.Generator(np.random.PCG64(seed))
    cfgs, conses = [], []
    for n in (32, 48, 64):
        gamma = float(rng.uniform(1.4, 5.0 / 3.0))
        cfg, cons = P.kh2d_smooth(n=n, block=16, ng=4 if recon == "ppm" else 2, recon=recon,
                                  rsolver="hllc", integrator="rk2", gamma=gamma)
        cfgs.append(cfg)
        conses.append(cons)
    return ensemble.Ensemble(cfgs, [1.0] * 3), conses


def test_ensemble_adjoint_matches_members_alone(cuda):
    """One batched reverse sweep over all members equals each member's own reverse sweep."""
    import torch
    from apophis_gb300.adjoint import Adjoint, EnsembleAdjoint
    ens, conses = _adjoint_ensemble()
    nsteps = 6
    dts = [[0.15 * c.dx[0] for c in ens.members] for _ in range(nsteps)]
    flat = torch.from_numpy(ens.pack(conses)).cuda()
    gen = torch.Generator(device="cuda").manual_seed(11)
    lam = torch.randn(flat.shape, dtype=torch.float64, device="cuda", generator=gen)
    ea = EnsembleAdjoint(ens)
    uT = ea.forward_members(flat, dts, checkpoint_every=4)
    lam0 = ea.backward(lam)
    uT_h, lam0_h = uT.cpu().numpy(), lam0.cpu().numpy()
    lam_h = lam.cpu().numpy()
    for m, cfg in enumerate(ens.members):
        a = Adjoint(cfg)
        u0m = torch.from_numpy(np.ascontiguousarray(conses[m])).cuda()
        uTm = a.forward(u0m, [r[m] for r in dts], 4)
        lm = torch.from_numpy(np.ascontiguousarray(ens.unpack(lam_h, m))).cuda()
        l0m = a.backward(lm)
        sk, sj, si = cfg.interior
        got_u = ens.unpack(uT_h, m)[:, :, sk, sj, si]
        want_u = uTm.cpu().numpy()[:, :, sk, sj, si]
        assert np.array_equal(got_u, want_u), m
        got = ens.unpack(lam0_h, m)
        want = l0m.cpu().numpy()
        err = np.abs(got - want).max() / np.abs(want).max()
        assert err <= 1e-13, (m, err)
        a.close()
    ea.close()


def test_ensemble_adjoint_member_finished_early(cuda):
    """A member past its end time (dt 0, its blocks skipped) while segments are recomputed:
    the batched reverse sweep stays finite and equals each member's own sweep over the steps
    it took (the skipped blocks' primitives include cells no pass ever formed)."""
    import torch
    from apophis_gb300.adjoint import Adjoint, EnsembleAdjoint
    ens, conses = _adjoint_ensemble(seed=5)
    nsteps, done0 = 6, 2
    dts = [[0.15 * c.dx[0] if (m > 0 or k < done0) else 0.0 for m, c in enumerate(ens.members)]
           for k in range(nsteps)]
    flat = torch.from_numpy(ens.pack(conses)).cuda()
    gen = torch.Generator(device="cuda").manual_seed(12)
    lam = torch.randn(flat.shape, dtype=torch.float64, device="cuda", generator=gen)
    ea = EnsembleAdjoint(ens)
    ea.forward_members(flat, dts, checkpoint_every=2)
    lam0_h = ea.backward(lam).cpu().numpy()
    lam_h = lam.cpu().numpy()
    assert np.isfinite(lam0_h).all()
    for m, cfg in enumerate(ens.members):
        a = Adjoint(cfg)
        u0m = torch.from_numpy(np.ascontiguousarray(conses[m])).cuda()
        steps = [r[m] for r in dts if r[m] > 0.0]
        a.forward(u0m, steps, 2)
        lm = torch.from_numpy(np.ascontiguousarray(ens.unpack(lam_h, m))).cuda()
        want = a.backward(lm).cpu().numpy()
        got = ens.unpack(lam0_h, m)
        sk, sj, si = cfg.interior
        err = np.abs(got[:, :, sk, sj, si] - want[:, :, sk, sj, si]).max() / np.abs(want).max()
        assert err <= 1e-13, (m, err)
        a.close()
    ea.close()


def test_ensemble_pressure_gradient_fd(cuda):
    """Gradient of L = sum_m ||rho_m(T)||^2 / 2 with respect to every member's initial pressure
    (one batched reverse sweep), against central differences on seeded directions.

    Donor-cell reconstruction, so that the step is smooth: this dL/dp is small (a cancelling
    sum, ~0.04 against ~170 for dL/drho), and limiter kinks that a step of h crosses spoil
    differences at the 1e-5..1e-4 level with PLM (the error falls with h until rounding takes
    over), while PPM's face and extremum limiters jump where a face value crosses a cell value.
    PLM and PPM are checked against the taped gradient instead."""
    import torch
    from apophis_gb300.adjoint import EnsembleAdjoint
    ens, conses = _adjoint_ensemble(seed=8, recon="dc")
    nsteps = 2
    dts = [[0.15 * c.dx[0] for c in ens.members] for _ in range(nsteps)]
    flat = torch.from_numpy(ens.pack(conses)).cuda()
    ea = EnsembleAdjoint(ens)

    def loss_of(u0):
        uT = ea.forward_members(u0, dts, checkpoint_every=2).cpu().numpy()
        tot = 0.0
        for m, cfg in enumerate(ens.members):
            sk, sj, si = cfg.interior
            r = ens.unpack(uT, m)[:, 0, sk, sj, si]
            tot += 0.5 * float((r ** 2).sum())
        return tot, uT

    L0, uT = loss_of(flat)
    lam = np.zeros_like(uT)
    for m, cfg in enumerate(ens.members):
        sk, sj, si = cfg.interior
        ens.unpack(lam, m)[:, 0, sk, sj, si] = ens.unpack(uT, m)[:, 0, sk, sj, si]
    lam0 = ea.backward(torch.from_numpy(lam).cuda()).cpu().numpy()
    # dE/dp = 1/gm1 at fixed rho and v: the pressure gradient is lam_E / gm1
    rng = np.random.Generator(np.random.PCG64(2))
    h = 1e-6
    for _ in range(4):
        dirs = np.zeros_like(lam0)
        pred = 0.0
        for m, cfg in enumerate(ens.members):
            sk, sj, si = cfg.interior
            d = rng.normal(size=ens.unpack(dirs, m)[:, 4, sk, sj, si].shape)
            ens.unpack(dirs, m)[:, 4, sk, sj, si] = d / cfg.gm1   # dE for dp = d
            pred += float((ens.unpack(lam0, m)[:, 4, sk, sj, si] / cfg.gm1 * d).sum())
        dflat = torch.from_numpy(dirs).cuda()
        # directional derivative of L through the state difference (no cancellation in L)
        _, up = loss_of(flat + h * dflat)
        _, um = loss_of(flat - h * dflat)
        fd = float((lam * (up - um)).sum()) / (2 * h)
        # HLLC's shock switch (p* = p) is a kink a step of 1e-6 crosses in a few faces:
        # agreement to ~1e-6 of this cancelling sum, bounded at 1e-5
        assert abs(fd - pred) <= 1e-5 * abs(pred), (fd, pred)
    ea.close()


def test_ensemble_tma_windows_match_plain_loads(cuda):
    """Equal blocks across members: the TMA-staged windows give the same bits (interiors:
    ghost cells hold stage inputs, which plain-load launches read at their sources)."""
    ens, conses, flat = small_ensemble()
    outs = []
    for tma in (0, 1):
        st = ensemble.EnsembleStepper(ens, flat, exact=False)
        c = dict(st.config, tma=tma, lines=[4, 4, 0])
        st.set_config(c)
        st.step(4)
        outs.append((st.state(), st.member_status()))
        st.close()
    assert outs[0][1] == outs[1][1]
    for m, cfg in enumerate(ens.members):
        sk, sj, si = cfg.interior
        a = ens.unpack(outs[0][0], m)[:, :, sk, sj, si]
        b = ens.unpack(outs[1][0], m)[:, :, sk, sj, si]
        assert np.array_equal(a, b), m
