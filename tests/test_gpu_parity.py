"""CUDA path vs the oracle, kernel by kernel and step by step (needs a GPU).

Both arithmetic modes are checked: exact must equal the oracle bit for bit, fast must
agree to the relative 1e-12 rule of parity_util.
"""
import numpy as np
import pytest
import torch

from apophis_gb300 import hydro
from oracle import oracle as O
from parity_util import assert_parity, interior_faces, l1_rel, small_workloads

pytestmark = pytest.mark.gpu

WORKLOADS = small_workloads()
IDS = [w[0] for w in WORKLOADS]


def _oracle_ready(cfg, cons):
    m = O.Mesh(cfg)
    m.set_cons(cons)  # fills ghosts, FillDerived, dt
    return m


@pytest.mark.parametrize("exact", [True, False], ids=["exact", "fast"])
@pytest.mark.parametrize("wl", WORKLOADS, ids=IDS)
def test_kernels_match_oracle(cuda, wl, exact):
    name, cfg, cons = wl
    m = _oracle_ready(cfg, cons)
    cons_g = m.get("cons")  # ghosts filled, floors applied
    prim_ref = m.get("prim")
    gamma_ref = m.get("gamma")
    md = hydro.MeshData(cfg, exact=exact)
    md.set_cons(cons_g)
    # ConsToPrim over the entire domain
    hydro.ConsToPrim(md)
    torch.cuda.synchronize()
    assert_parity(md.prim.cpu().numpy(), prim_ref, exact, what="prim")
    assert_parity(md.gamma.cpu().numpy(), gamma_ref, exact, what="gamma")
    # fluxes from identical inputs
    md.prim.copy_(torch.from_numpy(prim_ref))
    md.gamma.copy_(torch.from_numpy(gamma_ref))
    hydro.CalculateFluxes(md)
    torch.cuda.synchronize()
    nb = cfg.nblocks
    ref_flux = []
    for b in range(nb):
        fl = [np.zeros_like(cons_g[b]) for _ in range(3)]
        O.calculate_fluxes(np.ascontiguousarray(prim_ref[b]), np.ascontiguousarray(gamma_ref[b]),
                           fl, cfg.block_nx, cfg.ng, cfg.ndim, cfg.recon, cfg.rsolver)
        ref_flux.append(fl)
    for d in range(cfg.ndim):
        sl = (slice(None), slice(None)) + interior_faces(cfg, d)
        ref = np.stack([ref_flux[b][d] for b in range(nb)])[sl]
        assert_parity(md.flux[d].cpu().numpy()[sl], ref, exact, what="flux%d" % (d + 1), vector=True)
    # update from identical fluxes
    for d in range(cfg.ndim):
        md.flux[d].copy_(torch.from_numpy(np.stack([ref_flux[b][d] for b in range(nb)])))
    rng = np.random.default_rng(3)
    u1 = cons_g * (1.0 + 1e-3 * rng.standard_normal(cons_g.shape))
    md.u1.copy_(torch.from_numpy(u1))
    for gam0, gam1, beta in [(0.0, 1.0, 1.0), (0.5, 0.5, 0.5)]:
        md.cons.copy_(torch.from_numpy(cons_g))
        hydro.UpdateWithFluxDivergence(md, gam0, gam1, beta * 1.7e-3)
        torch.cuda.synchronize()
        ref = cons_g.copy()
        for b in range(nb):
            O.update(ref[b], np.ascontiguousarray(u1[b]), ref_flux[b], cfg.block_nx, cfg.ng,
                     cfg.ndim, cfg.dx, gam0, gam1, beta * 1.7e-3)
        assert_parity(md.cons.cpu().numpy(), ref, exact, what="update")
    # dt estimate
    md.cons.copy_(torch.from_numpy(cons_g))
    md.prim.copy_(torch.from_numpy(prim_ref))
    dt = hydro.EstimateTimestep(md)
    dt_ref = min(O.estimate_dt(np.ascontiguousarray(prim_ref[b]), np.ascontiguousarray(cons_g[b]),
                               cfg.block_nx, cfg.ng, cfg.ndim, cfg.dx, cfg.cfl, cfg.gm1)
                 for b in range(nb))
    if exact:
        assert dt == dt_ref
    else:
        assert abs(dt - dt_ref) <= 1e-13 * dt_ref


@pytest.mark.parametrize("per_block", [False, True], ids=["per_pack", "per_block"])
@pytest.mark.parametrize("exact", [True, False], ids=["exact", "fast"])
@pytest.mark.parametrize("wl", WORKLOADS, ids=IDS)
def test_rk_steps_match_oracle(cuda, wl, exact, per_block):
    """Three RK steps with the dt policy.  Exact: bit for bit every step.  Fast: 1e-12
    after the first step, then a loose L1 bound (see parity_util on limiter branches)."""
    name, cfg, cons = wl
    m = _oracle_ready(cfg, cons)
    drv = hydro.Driver(cfg, cons, exact=exact, per_block=per_block)
    if exact:
        assert drv.dt == m.state()["dt"]
    for step in range(3):
        m.run(nsteps=1)
        drv.run(nsteps=1)
        st = m.state()
        if exact:
            assert drv.dt == st["dt"], (step, drv.dt, st["dt"])
        else:
            assert abs(drv.dt - st["dt"]) <= 1e-12 * st["dt"]
        sk, sj, si = cfg.interior
        sl = (slice(None), slice(None), sk, sj, si)
        if exact or step == 0:
            assert_parity(drv.cons()[sl], m.get("cons")[sl], exact, what="cons step %d" % step)
        else:
            assert l1_rel(drv.cons()[sl], m.get("cons")[sl]) < 1e-6


def test_sod_full_run_l1(cuda):
    """Sod 1D (256 cells, PLM+HLLE, RK2, CFL 0.4) to t = 0.2: L1(rho) difference < 1e-10."""
    from apophis_gb300 import problems
    cfg, cons = problems.sod(nx=256, recon="plm", rsolver="hlle", integrator="rk2", cfl=0.4)
    m = _oracle_ready(cfg, cons)
    m.run(tlim=0.2)
    drv = hydro.Driver(cfg, cons, exact=False)
    drv.run(tlim=0.2)
    assert drv.ncycle == m.state()["ncycle"]
    g = cfg.ng
    rho_g = drv.cons()[0, 0, 0, 0, g:-g]
    rho_o = m.get("cons")[0, 0, 0, 0, g:-g]
    l1 = np.mean(np.abs(rho_g - rho_o))
    assert l1 < 1e-10, l1


@pytest.mark.parametrize("wl", [w for w in WORKLOADS if w[0] in ("sod_plm_hlle", "kh2d_ppm_hllc",
                                                                    "kh3d_ppm_hllc")],
                         ids=lambda w: w[0])
def test_face_centred_flux_arrays_and_eos_lambda(cuda, wl):
    """Parthenon's own field layout: flux arrays one face longer along their direction
    (passed with their strides) and the eos_lambda field.  ConsToPrim, CalculateFluxes and
    the update must give the oracle's bits (exact mode), the face arrays must hold the
    oracle's fluxes at every interior face, and eos_lambda's lT must become 7 as the
    reference's ConsToPrim makes it (hydro.cpp:491-493)."""
    name, cfg, cons = wl
    m = _oracle_ready(cfg, cons)
    cons_g, prim_ref, gamma_ref = m.get("cons"), m.get("prim"), m.get("gamma")
    md = hydro.MeshData(cfg, exact=True, face_fluxes=True, eos_lambda=True)
    for d in range(cfg.ndim):
        assert md.flux[d].shape[4 - d] == md.cons.shape[4 - d] + 1
    md.set_cons(cons_g)
    hydro.ConsToPrim(md)
    hydro.CalculateFluxes(md)
    torch.cuda.synchronize()
    assert_parity(md.prim.cpu().numpy(), prim_ref, True, what="prim")
    lam = md.eos_lambda.cpu().numpy()
    assert (lam[:, 2] == 7.0).all() and (lam[:, :2] == 0.0).all()
    nb = cfg.nblocks
    ref_flux = []
    for b in range(nb):
        fl = [np.zeros_like(cons_g[b]) for _ in range(3)]
        O.calculate_fluxes(np.ascontiguousarray(prim_ref[b]), np.ascontiguousarray(gamma_ref[b]),
                           fl, cfg.block_nx, cfg.ng, cfg.ndim, cfg.recon, cfg.rsolver)
        ref_flux.append(fl)
    nk, nj, ni = md.cons.shape[2:]
    for d in range(cfg.ndim):
        got = md.flux[d].cpu().numpy()[:, :, :nk, :nj, :ni]  # same (k, j, i) face indexing
        sl = (slice(None), slice(None)) + interior_faces(cfg, d)
        ref = np.stack([ref_flux[b][d] for b in range(nb)])[sl]
        assert_parity(got[sl], ref, True, what="flux%d" % (d + 1))
    u1 = cons_g.copy()
    md.u1.copy_(torch.from_numpy(u1))
    hydro.UpdateWithFluxDivergence(md, 0.5, 0.5, 1.3e-3)
    torch.cuda.synchronize()
    ref = cons_g.copy()
    for b in range(nb):
        O.update(ref[b], np.ascontiguousarray(u1[b]), ref_flux[b], cfg.block_nx, cfg.ng, cfg.ndim,
                 cfg.dx, 0.5, 0.5, 1.3e-3)
    sk, sj, si = cfg.interior
    sl = (slice(None), slice(None), sk, sj, si)
    assert_parity(md.cons.cpu().numpy()[sl], ref[sl], True, what="update")
    md.close()
