"""Blocks where the pressure floor fires (ConsToPrim, hydro.cpp:485-505): the fast mode then
reconstructs the adiabatic-index fields instead of using the gas constants, in smaller line
chunks of a pass item.  Parity with the oracle in both modes, and bit-identical results
across line counts (chunk boundaries)."""
import numpy as np
import pytest

from apophis_gb300 import hydro, problems
from apophis_gb300.stepper import Stepper
from oracle import oracle as O
from parity_util import assert_parity

pytestmark = pytest.mark.gpu

METHODS = [("ppm", "hllc", 3), ("plm", "hlle", 2), ("ppm", "lhllc", 4)]


def _interior(cfg, a):
    sk, sj, si = cfg.interior
    return a[:, :, sk, sj, si]


def _floored_state(recon, rsolver, ng, steps=4):
    """The oracle's state after `steps` steps: the floor fires at its next ConsToPrim."""
    cfg, cons = problems.rarefaction2d(recon=recon, rsolver=rsolver, ng=ng)
    m = O.Mesh(cfg)
    m.set_cons(cons)
    m.run(nsteps=steps)
    return cfg, m.get("cons")


@pytest.mark.parametrize("recon,rsolver,ng", METHODS)
def test_floors_exact_run_matches_oracle(cuda, recon, rsolver, ng):
    cfg, cons = problems.rarefaction2d(recon=recon, rsolver=rsolver, ng=ng)
    m = O.Mesh(cfg)
    m.set_cons(cons)
    st = Stepper(cfg, cons, exact=True)
    d = hydro.Driver(cfg, cons, exact=True)
    for _ in range(7):
        m.run(nsteps=1)
        st.step(1)
        d.run(nsteps=1)
        want = _interior(cfg, m.get("cons"))
        assert st.status()["dt"] == m.state()["dt"]
        assert np.array_equal(_interior(cfg, st.state()), want)
        assert np.array_equal(_interior(cfg, d.cons()), want)
    d.md.close()
    st.close()


@pytest.mark.parametrize("recon,rsolver,ng", METHODS)
def test_floors_fast_step_matches_oracle(cuda, recon, rsolver, ng):
    cfg, cons = _floored_state(recon, rsolver, ng)
    m = O.Mesh(cfg)
    m.set_cons(cons)
    m.run(nsteps=1)
    want = _interior(cfg, m.get("cons"))
    for lines in ([2, 2, 0], [6, 6, 0], [16, 16, 0]):
        st = Stepper(cfg, cons, exact=False)
        c = st.config
        c.update(lines=lines)
        st.set_config(c)
        st.step(1)
        assert_parity(_interior(cfg, st.state()), want, False, what="cons")
        st.close()
    d = hydro.Driver(cfg, cons, exact=False)
    d.run(nsteps=1)
    assert_parity(_interior(cfg, d.cons()), want, False, what="cons")
    d.md.close()


def test_floors_fast_bit_identical_across_line_counts(cuda):
    """Items of floored blocks split into chunks of fewer lines: the same cells, same bits."""
    cfg, cons = _floored_state("ppm", "hllc", 3)
    outs = []
    for threads in (128, 256):
        for lines in ([1, 1, 0], [3, 5, 0], [6, 6, 0], [7, 7, 0], [16, 16, 0]):
            st = Stepper(cfg, cons, exact=False)
            c = st.config
            c.update(lines=lines, threads=threads)
            st.set_config(c)
            st.step(4)
            outs.append((st.state(), st.status()))
            st.close()
    for out, status in outs[1:]:
        assert np.array_equal(out, outs[0][0]) and status == outs[0][1]


def test_floors_with_face_tables_exact(cuda):
    """Floors firing on a pack described by face tables (the refined-mesh ghost map, here on an
    unrefined mesh): the batched stepper stays bit-identical to the refined-mesh oracle, which
    equals the uniform one."""
    from apophis_gb300 import amr
    cfg, cons = problems.rarefaction2d()
    acfg = amr.uniform_as_amr(cfg)
    flat = np.ascontiguousarray(cons).reshape(-1)
    m = O.AmrMesh(acfg)
    m.set_cons(flat)
    st = amr.AmrStepper(acfg, flat, exact=True)
    ng = acfg.ng
    for _ in range(6):
        m.run(nsteps=1)
        st.step(1)
        got, want = st.state(), m.get()
        for b in range(acfg.nblocks):
            assert np.array_equal(acfg.block_view(got, b)[:, 0, ng:-ng, ng:-ng],
                                  acfg.block_view(want, b)[:, 0, ng:-ng, ng:-ng]), b
    st.close()
