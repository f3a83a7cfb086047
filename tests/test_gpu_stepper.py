"""The batched stepper (one persistent launch per stage, graph-replayed steps) against
the oracle, plus its launch configuration, autotuner and error handling (needs a GPU)."""
import numpy as np
import pytest

from apophis_gb300 import problems
from apophis_gb300.stepper import Stepper
from oracle import oracle as O
from parity_util import assert_parity, l1_rel, small_workloads

pytestmark = pytest.mark.gpu

WORKLOADS = small_workloads()
IDS = [w[0] for w in WORKLOADS]


def _interior(cfg, a):
    sk, sj, si = cfg.interior
    return a[:, :, sk, sj, si]


@pytest.mark.parametrize("exact", [True, False], ids=["exact", "fast"])
@pytest.mark.parametrize("wl", WORKLOADS, ids=IDS)
def test_stepper_matches_oracle(cuda, wl, exact):
    name, cfg, cons = wl
    m = O.Mesh(cfg)
    m.set_cons(cons)
    st = Stepper(cfg, cons, exact=exact)
    s0 = st.status()
    if exact:
        assert s0["dt"] == m.state()["dt"]
    for step in range(3):
        m.run(nsteps=1)
        st.step(1)
        s = st.status()
        ref = m.state()
        assert s["ncycle"] == ref["ncycle"]
        if exact:
            assert s["dt"] == ref["dt"] and s["time"] == ref["time"]
            assert_parity(_interior(cfg, st.state()), _interior(cfg, m.get("cons")), True,
                          what="cons step %d" % step)
        else:
            assert abs(s["dt"] - ref["dt"]) <= 1e-12 * ref["dt"]
            if step == 0:
                assert_parity(_interior(cfg, st.state()), _interior(cfg, m.get("cons")), False)
            else:
                assert l1_rel(_interior(cfg, st.state()), _interior(cfg, m.get("cons"))) < 1e-6
    st.close()


@pytest.mark.parametrize("integ", ["rk1", "rk3", "vl2"])
def test_stepper_integrators_exact(cuda, integ):
    cfg, cons = problems.kh2d(n=32, block=16, ng=3, recon="ppm", rsolver="hllc",
                              integrator=integ)
    m = O.Mesh(cfg)
    m.set_cons(cons)
    st = Stepper(cfg, cons, exact=True)
    m.run(nsteps=3)
    st.step(3)
    assert st.status()["dt"] == m.state()["dt"]
    assert_parity(_interior(cfg, st.state()), _interior(cfg, m.get("cons")), True)


def test_stepper_sod_to_tlim(cuda):
    """Sod 1D (256 cells, PLM+HLLE) to t = 0.2 in the batched path, L1(rho) vs oracle < 1e-10."""
    cfg, cons = problems.sod(nx=256, recon="plm", rsolver="hlle", integrator="rk2", cfl=0.4)
    m = O.Mesh(cfg)
    m.set_cons(cons)
    m.run(tlim=0.2)
    st = Stepper(cfg, cons, exact=False, tlim=0.2)
    s = st.run(tlim=0.2)
    assert s["ncycle"] == m.state()["ncycle"]
    assert abs(s["time"] - 0.2) < 1e-14
    g = cfg.ng
    l1 = np.mean(np.abs(st.state()[0, 0, 0, 0, g:-g] - m.get("cons")[0, 0, 0, 0, g:-g]))
    assert l1 < 1e-10


def test_stepper_configs_agree(cuda):
    """Every schedule / CTA size / lines-per-item choice gives the same bits (exact)."""
    cfg, cons = problems.kh3d(n=16, block=8, ng=4)
    ref = None
    for cfgd in [dict(threads=256, schedule=0, lines=[0, 0, 0]),
                 dict(threads=128, schedule=1, lines=[3, 5, 2]),
                 dict(threads=256, schedule=2, lines=[1, 1, 1]),
                 dict(threads=256, schedule=2, lines=[2, 3, 1], reg_cap=1)]:
        st = Stepper(cfg, cons, exact=True)
        c = st.config
        c.update(cfgd)
        st.set_config(c)
        st.step(2)
        out = _interior(cfg, st.state())
        if ref is None:
            ref = out
        else:
            assert np.array_equal(out, ref)
        st.close()


def test_stepper_sweep_order_fast(cuda):
    cfg, cons = problems.kh3d(n=16, block=8, ng=4)
    m = O.Mesh(cfg)
    m.set_cons(cons)
    m.run(nsteps=1)
    st = Stepper(cfg, cons, exact=False)
    c = st.config
    c["order"] = [3, 1, 2]
    st.set_config(c)
    st.step(1)
    assert_parity(_interior(cfg, st.state()), _interior(cfg, m.get("cons")), False)
    st2 = Stepper(cfg, cons, exact=True)
    c = st2.config
    c["order"] = [2, 1, 3]
    with pytest.raises(Exception):
        st2.set_config(c)


def test_stepper_autotune_keeps_state(cuda, tmp_path):
    cfg, cons = problems.kh2d(n=64, block=32, ng=3, recon="ppm", rsolver="hllc")
    m = O.Mesh(cfg)
    m.set_cons(cons)
    m.run(nsteps=2)
    st = Stepper(cfg, cons, exact=True)
    rec = st.autotune(trial_steps=1, cache=str(tmp_path / "tune.json"))
    assert rec["ms_per_step"] > 0
    assert st.status()["ncycle"] == 0
    st.step(2)
    assert_parity(_interior(cfg, st.state()), _interior(cfg, m.get("cons")), True)
    # the cached record is reused
    st2 = Stepper(cfg, cons, exact=True)
    rec2 = st2.autotune(trial_steps=1, cache=str(tmp_path / "tune.json"))
    assert rec2["config"] == rec["config"]


@pytest.mark.parametrize("make,lines", [
    (lambda: problems.kh3d(n=16, block=8, ng=4), [2, 2, 2]),
    (lambda: problems.kh3d(n=16, block=8, ng=4), [4, 4, 4]),
    (lambda: problems.kh2d(n=64, block=32, ng=4, recon="ppm", rsolver="hllc"), [4, 8, 0]),
    (lambda: problems.kh2d(n=64, block=32, ng=2, recon="plm", rsolver="hlle"), [2, 2, 0]),
    # items crossing a plane of lines (two tensor copies)
    (lambda: problems.kh3d(n=16, block=8, ng=4), [6, 6, 6]),
    (lambda: problems.kh2d(n=64, block=32, ng=4, recon="ppm", rsolver="hllc"), [6, 6, 0]),
])
def test_stepper_tma_windows_match_plain_loads(cuda, make, lines):
    """TMA-staged windows change only how prim reaches shared memory: bit-identical steps."""
    cfg, cons = make()
    outs = []
    for tma in (0, 1):
        for reg_cap in (0, 1):
            st = Stepper(cfg, cons, exact=False)
            c = st.config
            c.update(lines=lines, tma=tma, reg_cap=reg_cap, schedule=2)
            st.set_config(c)
            st.step(3)
            sk, sj, si = cfg.interior  # ghost cells hold stage inputs, not the state
            outs.append((st.state()[:, :, sk, sj, si], st.status()))
            st.close()
    for out, status in outs[1:]:
        assert np.array_equal(out, outs[0][0]) and status == outs[0][1]


@pytest.mark.parametrize("where", ["device", "pinned", "pageable"])
def test_stepper_interiors_round_trip(cuda, where):
    """Packed interiors out and back in: the same bits, from device, pinned and pageable memory."""
    import torch
    cfg, cons = problems.kh3d(n=16, block=8, ng=4)
    st = Stepper(cfg, cons, exact=True)
    st.step(2)
    shape = st.interior_shape()
    if where == "device":
        buf = torch.empty(shape, dtype=torch.float64, device="cuda")
    elif where == "pinned":
        buf = torch.empty(shape, dtype=torch.float64, pin_memory=True)
    else:
        buf = np.empty(shape)
    st.store_interiors(buf)
    torch.cuda.synchronize()
    got = buf.cpu().numpy() if isinstance(buf, torch.Tensor) else buf
    assert np.array_equal(got, _interior(cfg, st.state()))
    # load a different state: the state's interiors are its values; it steps
    new = _interior(cfg, cons).copy()
    new[:, 4] *= 1.01
    if isinstance(buf, torch.Tensor):
        buf.copy_(torch.as_tensor(new))
    else:
        buf[...] = new
    st.load_interiors(buf)
    assert np.array_equal(_interior(cfg, st.state()), new)
    st.step(1)
    st.status()
    st.close()


def test_stepper_interiors_round_trip_keeps_floors(cuda):
    """Storing and loading back between steps leaves the run bit-identical, floors included."""
    import torch
    cfg, cons = problems.rarefaction2d()
    a = Stepper(cfg, cons, exact=True)
    b = Stepper(cfg, cons, exact=True)
    buf = torch.empty(b.interior_shape(), dtype=torch.float64, pin_memory=True)
    for _ in range(7):
        a.step(1)
        b.step(1)
        b.store_interiors(buf)
        b.load_interiors(buf)
    assert np.array_equal(_interior(cfg, a.state()), _interior(cfg, b.state()))
    a.close()
    b.close()
