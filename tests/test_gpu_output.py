"""The reference's Sod analysis (riemann_hydro.py:115-156) re-run on a dump written from the
GPU path and read back through the phdf-like reader."""
import json
import os

import numpy as np
import pytest

from apophis_gb300 import output, problems
from apophis_gb300.stepper import Stepper

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_sod_dump_reanalysed(cuda, tmp_path):
    pins = json.load(open(os.path.join(GOLD, "pins.json")))
    ex = np.loadtxt(os.path.join(GOLD, "sod_exact_t0245.txt"))
    cfg, cons = problems.sod(nx=128, x0=1.0, xmin=0.0, xmax=2.0, recon="plm", rsolver="hllc",
                             integrator="vl2", cfl=0.5)
    st = Stepper(cfg, cons, tlim=pins["sod_tlim"])
    st.run(tlim=pins["sod_tlim"])
    s = st.status()
    state = st.state()
    # primitives of the final state (the dump carries what phdf's "prim" holds)
    prim = np.zeros_like(state)
    rho = state[:, 0]
    prim[:, 0] = rho
    prim[:, 1:4] = state[:, 1:4] / rho[:, None]
    prim[:, 4] = cfg.gm1 * (state[:, 4] - 0.5 * (state[:, 1:4] ** 2).sum(axis=1) / rho)
    base = str(tmp_path / "sod.final")
    output.write_dump(base, cfg, state, s["time"], s["ncycle"], prim=prim)
    st.close()

    d = output.Dump(base)
    assert d.Time == pytest.approx(pins["sod_tlim"], abs=1e-15)
    p = d.Get("prim")[0]           # block 0: (cells, nvar), as the reference indexes it
    rho, vx, pres = p[:, 0], p[:, 1], p[:, 4]
    zz, yy, xx = d.GetVolumeLocations()
    xx = xx[0]
    rho_ex = np.interp(xx, ex[:, 0], ex[:, 1])
    v_ex = np.interp(xx, ex[:, 0], ex[:, 2])
    p_ex = np.interp(xx, ex[:, 0], ex[:, 3])
    thr = pins["sod_exact_threshold"]
    assert np.max(rho_ex - rho) <= thr and np.max(p_ex - pres) <= thr
    assert np.mean(np.abs(v_ex - vx)) < 0.01
    # the dump round-trips the state exactly
    sk, sj, si = cfg.interior
    assert np.array_equal(d.Get("cons", flatten=False), state[:, :, sk, sj, si])
