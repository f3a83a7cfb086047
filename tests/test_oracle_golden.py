"""Pin the oracle against the reference's own golden data and known answers.

* the exact Sod solution embedded in the reference's riemann_hydro test
  (tst/regression/test_suites/riemann_hydro/riemann_hydro.py:115-156, 192-272);
* the linear-wave RMS-L1 bound of the reference's convergence test
  (tst/regression/test_suites/convergence/convergence.py:130);
* known answers of the reconstructions and Riemann solvers.
"""
import json
import os

import numpy as np
import pytest

from apophis_gb300 import problems
from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden")
PINS = json.load(open(os.path.join(GOLD, "pins.json")))

# riemann_hydro.py:17-23 (nx1 = 128 on [0, 2], interface at x = 1, cfl 0.5 from sod.in)
SOD_METHODS = [("vl2", "plm", "hlle"), ("vl2", "plm", "hllc"), ("rk2", "plm", "hllc"),
               ("rk3", "plm", "hlle"), ("rk3", "plm", "hllc")]


@pytest.mark.parametrize("integ,recon,rs", SOD_METHODS)
def test_sod_matches_reference_exact_solution(integ, recon, rs):
    ex = np.loadtxt(os.path.join(GOLD, "sod_exact_t0245.txt"))
    cfg, cons = problems.sod(nx=128, x0=1.0, xmin=0.0, xmax=2.0, recon=recon, rsolver=rs,
                             integrator=integ, cfl=0.5)
    m = O.Mesh(cfg)
    m.set_cons(cons)
    m.run(tlim=PINS["sod_tlim"])
    assert abs(m.state()["time"] - PINS["sod_tlim"]) < 1e-15
    g = cfg.ng
    w = m.get("prim")[0][:, 0, 0, g:-g]
    x = cfg.cell_centers(0)[0][0, 0]
    rho_ex = np.interp(x, ex[:, 0], ex[:, 1])
    v_ex = np.interp(x, ex[:, 0], ex[:, 2])
    p_ex = np.interp(x, ex[:, 0], ex[:, 3])
    thr = PINS["sod_exact_threshold"]
    # the reference's own (one-sided) check, riemann_hydro.py:147-151, for rho and p
    assert np.max(rho_ex - w[0]) <= thr
    assert np.max(p_ex - w[4]) <= thr
    # velocity: the reference only prints this check; its smeared shock front exceeds
    # 0.05 in one or two cells for every method, so bound the L1 error instead
    assert np.mean(np.abs(v_ex - w[1])) < 0.01
    assert np.mean(np.abs(rho_ex - w[0])) < 0.005


@pytest.mark.slow
def test_linear_wave_convergence_pin():
    """convergence.py:130: RMS-L1 error of vl2+plm+hllc at 128x64x64 <= 4.63e-8."""
    lw = problems.LinearWave(res=64, recon="plm", rsolver="hllc", integrator="vl2")
    m = O.Mesh(lw.cfg)
    m.set_cons(lw.solution())
    m.run(tlim=lw.tlim)
    err, _ = lw.rms_l1_error(m.get("cons"))
    assert err <= PINS["linear_wave_rms_l1_max"]


def test_linear_wave_second_order():
    errs = []
    for res in (16, 32):
        lw = problems.LinearWave(res=res, recon="plm", rsolver="hllc", integrator="rk2")
        m = O.Mesh(lw.cfg)
        m.set_cons(lw.solution())
        m.run(tlim=lw.tlim)
        errs.append(lw.rms_l1_error(m.get("cons"))[0])
    assert errs[0] / errs[1] > 2.5


def test_reconstruction_known_answers():
    # constants are reproduced exactly
    for c in (0.0, 1.0, -3.25, 1e-300):
        assert O.plm(c, c, c) == (c, c)
        assert O.ppm(c, c, c, c, c) == (c, c)
    # linear data: PLM face values are the linear interpolant, PPM too
    ql, qr = O.plm(1.0, 2.0, 3.0)
    assert (ql, qr) == (2.5, 1.5)
    ql, qr = O.ppm(0.0, 1.0, 2.0, 3.0, 4.0)
    assert abs(ql - 2.5) < 1e-15 and abs(qr - 1.5) < 1e-15
    # extremum: PLM flattens
    assert O.plm(1.0, 2.0, 1.0) == (2.0, 2.0)


@pytest.mark.parametrize("rs", ["hlle", "hllc", "lhllc"])
def test_riemann_identical_states_give_physical_flux(rs):
    gamma = 1.4
    rng = np.random.default_rng(1)
    for _ in range(20):
        rho, p = rng.uniform(0.1, 3.0, 2)
        v = rng.uniform(-1.0, 1.0, 3)
        if rs == "lhllc":
            v *= 0.05
        w = np.array([rho, v[0], v[1], v[2], p])
        g = np.array([gamma, gamma])
        f = O.riemann(rs, w, w, g, g)
        e = p / (gamma - 1) + 0.5 * rho * np.dot(v, v)
        phys = np.array([rho * v[0], rho * v[0] ** 2 + p, rho * v[0] * v[1], rho * v[0] * v[2],
                         (e + p) * v[0]])
        np.testing.assert_allclose(f, phys, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("rs", ["hlle", "hllc"])
def test_riemann_mirror_symmetry(rs):
    rng = np.random.default_rng(2)
    g = np.array([1.4, 1.4])
    for _ in range(20):
        wl = np.array([*rng.uniform(0.2, 2.0, 1), *rng.uniform(-1, 1, 3), *rng.uniform(0.2, 2.0, 1)])
        wr = np.array([*rng.uniform(0.2, 2.0, 1), *rng.uniform(-1, 1, 3), *rng.uniform(0.2, 2.0, 1)])
        f = O.riemann(rs, wl, wr, g, g)
        ml = wr.copy(); ml[1] = -ml[1]
        mr = wl.copy(); mr[1] = -mr[1]
        fm = O.riemann(rs, ml, mr, g, g)
        # x -> -x: mass, transverse momenta and energy flux flip sign, normal momentum flux does not
        np.testing.assert_allclose(fm[[0, 2, 3, 4]], -f[[0, 2, 3, 4]], rtol=1e-12, atol=1e-13)
        np.testing.assert_allclose(fm[1], f[1], rtol=1e-12, atol=1e-13)
