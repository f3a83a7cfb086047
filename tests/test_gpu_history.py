"""History sums (GlobalQuantHst: total_mass, total_energy) of the per-kernel pack and the
batched stepper against the oracle's sums, their determinism, and conservation."""
import numpy as np
import pytest

from apophis_gb300 import hydro, problems
from apophis_gb300.stepper import Stepper
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("make", [lambda: problems.kh3d(n=32, block=16, ng=4),
                                  lambda: problems.rt2d(nx=32, ny=96, block=(16, 16))])
def test_pack_history_matches_oracle(cuda, make):
    cfg, cons = make()
    md = hydro.MeshData(cfg)
    md.set_cons(cons)
    got = hydro.History(md)
    want = O.history(cfg, cons)
    for k in ("total_mass", "total_energy"):
        assert got[k] == pytest.approx(want[k], rel=1e-14, abs=0), k
    assert hydro.History(md) == got  # fixed reduction order: bit-identical on repeat
    md.close()


def test_stepper_history_conserved(cuda):
    cfg, cons = problems.kh3d(n=32, block=16, ng=4)
    st = Stepper(cfg, cons)
    h0 = st.history()
    want0 = O.history(cfg, cons)
    assert h0["total_mass"] == pytest.approx(want0["total_mass"], rel=1e-14)
    st.step(10)
    h1 = st.history()
    # periodic box: mass and energy are conserved to round-off
    assert abs(h1["total_mass"] - h0["total_mass"]) <= 1e-13 * h0["total_mass"]
    assert abs(h1["total_energy"] - h0["total_energy"]) <= 1e-13 * h0["total_energy"]
    # and equal the oracle's sums of the stepper's state
    want1 = O.history(cfg, st.state())
    assert h1["total_mass"] == pytest.approx(want1["total_mass"], rel=1e-14)
    assert h1["total_energy"] == pytest.approx(want1["total_energy"], rel=1e-14)
    st.close()
