"""Passive scalars (hydro/composition; fluxes upwinded by the mass flux, hydro.cpp:607-615)
on the per-kernel path: every step bit-identical to the oracle in exact mode, 1e-12 in fast
mode, tracer mass conserved."""
import numpy as np
import pytest

from apophis_gb300 import hydro, problems
from oracle import oracle as O
from parity_util import assert_parity

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("recon,rsolver", [("plm", "hllc"), ("ppm", "hlle"), ("dc", "hlle")])
@pytest.mark.parametrize("per_block", [False, True], ids=["per_pack", "per_block"])
def test_scalars_match_oracle(cuda, recon, rsolver, per_block):
    ng = 3 if recon == "ppm" else 2
    cfg, cons = problems.kh2d_tracers(n=48, block=16, ng=ng, recon=recon, rsolver=rsolver)
    assert cfg.nvar == 7
    for exact in (True, False):
        nsteps = 3 if exact else 1
        m = O.Mesh(cfg)
        m.set_cons(cons)
        m.run(nsteps=nsteps)
        d = hydro.Driver(cfg, cons, exact=exact, per_block=per_block)
        d.run(nsteps=nsteps)
        assert d.time == m.state()["time"] or not exact
        sk, sj, si = cfg.interior
        got = d.cons()[:, :, sk, sj, si]
        want = m.get("cons")[:, :, sk, sj, si]
        assert_parity(got, want, exact, what="cons")
        d.md.close()


def test_tracer_mass_conserved(cuda):
    cfg, cons = problems.kh2d_tracers(n=64, block=32, ng=2)
    d = hydro.Driver(cfg, cons, exact=False)
    d.run(nsteps=20)
    sk, sj, si = cfg.interior
    out = d.cons()
    for k in range(cfg.nscalars):
        before = cons[:, 5 + k][:, sk, sj, si].sum()
        after = out[:, 5 + k][:, sk, sj, si].sum()
        assert abs(after - before) <= 1e-12 * abs(before)
    d.md.close()
