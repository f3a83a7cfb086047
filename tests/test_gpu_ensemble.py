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
