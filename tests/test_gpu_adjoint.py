"""The hand-written adjoint of the hydro step (needs a GPU).

* one-step vector-Jacobian products against the taped reference gradient of a PyTorch
  FP64 restatement of the same step (torch.autograd);
* checkpointed rollouts wrapped in a torch.autograd.Function (here, in the tests only),
  loss || rho(T) - rho_target ||_2 with respect to the initial density and v_y, against the
  taped gradient of the restated rollout and against central finite differences on 32
  seeded random directions;
* checkpoint spacing does not change the gradient.

Finite differences and the limiter's kinks: the PLM limiter of plm_simple.hpp:15-32 has a
kink wherever a field has a local extremum (dq2 = dql*dqr changes sign) and the HLLE
shock branch one where p_mid = p.  A perturbation of 1e-6 per cell crosses such kinks in
~1e-3 of the cells of a KH flow, so central differences with step 1e-6 agree with the
*exact* gradient of the scheme only to ~1e-3 (measured on the taped restatement: median
2e-3 after one step, 1e-3 after twenty); with step 1e-8 they agree to ~1e-7 after one step.
The tests therefore check the adjoint tightly against the taped gradient, against
differences with step 1e-8 on one step, and against differences with the prescribed step
1e-6 to within what the exact taped gradient itself achieves.
"""
import numpy as np
import pytest
import torch

import torch_reference as TR
from apophis_gb300 import problems
from apophis_gb300.adjoint import Adjoint

pytestmark = pytest.mark.gpu


def pack_from_global(cfg, G):
    out = torch.zeros(cfg.pack_shape(5), dtype=G.dtype, device=G.device)
    sk, sj, si = cfg.interior
    bn = cfg.block_nx
    for b in range(cfg.nblocks):
        bi, bj, bk = cfg.block_index(b)
        out[b, :, sk, sj, si] = G[:, bk * bn[2]:(bk + 1) * bn[2], bj * bn[1]:(bj + 1) * bn[1],
                                  bi * bn[0]:(bi + 1) * bn[0]]
    return out


def global_from_pack(cfg, P):
    sk, sj, si = cfg.interior
    nb = cfg.blocks_per_dim
    bn = cfg.block_nx
    inner = P[:, :, sk, sj, si]  # (nblocks, 5, n3, n2, n1)
    x = inner.reshape(nb[2], nb[1], nb[0], 5, bn[2], bn[1], bn[0])
    x = x.permute(3, 0, 4, 1, 5, 2, 6)
    return x.reshape(5, nb[2] * bn[2], nb[1] * bn[1], nb[0] * bn[0])


class Rollout(torch.autograd.Function):
    """u0 (pack) -> u(T) through the C ABI; backward through the hand-written adjoint."""

    @staticmethod
    def forward(ctx, u0, adj, dts, ckpt):
        ctx.adj = adj
        return adj.forward(u0.detach().contiguous(), dts, ckpt)

    @staticmethod
    def backward(ctx, g):
        return ctx.adj.backward(g.contiguous()), None, None, None


def kh_setup(n, block, rs, integ, recon="plm"):
    cfg, cons = problems.kh2d_smooth(n=n, block=block, ng=4 if recon == "ppm" else 2, recon=recon,
                                     rsolver=rs, integrator=integ)
    return cfg, torch.from_numpy(cons).cuda()


@pytest.mark.parametrize("rs,integ,recon", [("hlle", "rk2", "plm"), ("hllc", "rk2", "plm"),
                                            ("hlle", "vl2", "plm"), ("hllc", "rk3", "plm"),
                                            ("hlle", "rk1", "dc"), ("hllc", "rk2", "ppm"),
                                            ("hlle", "rk3", "ppm")])
def test_step_vjp_matches_taped_reference(cuda, rs, integ, recon):
    cfg, u = kh_setup(64, 32, rs, integ, recon)
    adj = Adjoint(cfg)
    dt = 2e-3
    # forward agrees with the torch restatement
    G = global_from_pack(cfg, u).requires_grad_(True)
    ref_next = TR.step(G, dt, cfg.dx, cfg.gamma, cfg.recon, cfg.rsolver, cfg.integrator, cfg.ndim)
    got_next = global_from_pack(cfg, adj.step(u, dt))
    assert torch.allclose(got_next, ref_next.detach(), rtol=1e-12, atol=1e-13)
    # vjp agrees with torch.autograd through the restatement
    gen = torch.Generator(device="cuda").manual_seed(7)
    lamG = torch.randn(ref_next.shape, dtype=torch.float64, device="cuda", generator=gen)
    (ref_vjp,) = torch.autograd.grad(ref_next, G, lamG)
    got_vjp = global_from_pack(cfg, adj.step_vjp(u, dt, pack_from_global(cfg, lamG)))
    err = (got_vjp - ref_vjp).norm() / ref_vjp.norm()
    assert err < 1e-11, float(err)
    # ghost entries of the adjoint output are zero
    out = adj.step_vjp(u, dt, pack_from_global(cfg, lamG))
    mask = torch.ones_like(out, dtype=torch.bool)
    sk, sj, si = cfg.interior
    mask[:, :, sk, sj, si] = False
    assert float(out[mask].abs().max()) == 0.0


def _loss_and_grad(cfg, adj, rho0, vy0, base_prim, dts, ckpt, target, need_grad=True):
    W = base_prim.clone()
    W[0] = rho0
    W[2] = vy0
    U = TR.prim_to_cons(W, cfg.gm1)
    u_T = Rollout.apply(pack_from_global(cfg, U), adj, dts, ckpt)
    rho_T = global_from_pack(cfg, u_T)[0]
    loss = torch.sqrt(torch.sum((rho_T - target) ** 2))
    if not need_grad:
        return float(loss)
    gr, gv = torch.autograd.grad(loss, (rho0, vy0))
    return float(loss), gr, gv


def _setup_rollout(cfg, nsteps, seed):
    _, cons = problems.kh2d_smooth(n=cfg.mesh_nx[0], block=cfg.block_nx[0], ng=cfg.ng,
                                   recon=cfg.recon, rsolver=cfg.rsolver,
                                   integrator=cfg.integrator)
    U0 = global_from_pack(cfg, torch.from_numpy(cons).cuda())
    W0 = TR.c2p(U0, cfg.gm1)
    # fixed dt schedule: the CFL estimate of the initial state, held constant
    dt = 0.3 * 0.5 * cfg.dx[0] / float((W0[1].abs() + torch.sqrt(cfg.gamma * W0[4] / W0[0])).max())
    dts = [dt] * nsteps
    gen = torch.Generator(device="cuda").manual_seed(seed)
    Wt = W0.clone()
    Wt[2] = Wt[2] + 1e-3 * torch.randn(Wt[2].shape, dtype=torch.float64, device="cuda", generator=gen)
    return W0, Wt, dts, gen


def _fd_rel(cfg, adj, W0, dts, ckpt, tgt, gr, gv, h, ndir, gen):
    errs = []
    for _ in range(ndir):
        dr = torch.randn(gr.shape, dtype=torch.float64, device="cuda", generator=gen)
        dv = torch.randn(gv.shape, dtype=torch.float64, device="cuda", generator=gen)
        with torch.no_grad():
            lp = _loss_and_grad(cfg, adj, W0[0] + h * dr, W0[2] + h * dv, W0, dts, ckpt, tgt, False)
            lm = _loss_and_grad(cfg, adj, W0[0] - h * dr, W0[2] - h * dv, W0, dts, ckpt, tgt, False)
        fd = (lp - lm) / (2 * h)
        an = float((gr * dr).sum() + (gv * dv).sum())
        errs.append(abs(fd - an) / max(abs(fd), abs(an), 1e-300))
    return np.array(errs)


def _taped_grad(cfg, W0, dts, tgt):
    rho0 = W0[0].clone().requires_grad_(True)
    vy0 = W0[2].clone().requires_grad_(True)
    W = W0.clone()
    W[0] = rho0
    W[2] = vy0
    U = TR.prim_to_cons(W, cfg.gm1)
    for dt in dts:
        U = TR.step(U, dt, cfg.dx, cfg.gamma, cfg.recon, cfg.rsolver, cfg.integrator, cfg.ndim)
    loss = torch.sqrt(torch.sum((U[0] - tgt) ** 2))
    return torch.autograd.grad(loss, (rho0, vy0))


@pytest.mark.parametrize("rs", ["hlle", "hllc"])
def test_rollout_gradient_matches_taped_reference(cuda, rs):
    """20 steps, a checkpoint every 5: the checkpointed adjoint equals torch.autograd through
    the restated rollout."""
    cfg, _ = kh_setup(64, 32, rs, "rk2")
    adj = Adjoint(cfg)
    W0, Wt, dts, gen = _setup_rollout(cfg, 20, seed=11)
    with torch.no_grad():
        tgt = global_from_pack(cfg, adj.forward(pack_from_global(cfg, TR.prim_to_cons(Wt, cfg.gm1)), dts, 5))[0]
    rho0 = W0[0].clone().requires_grad_(True)
    vy0 = W0[2].clone().requires_grad_(True)
    _, gr, gv = _loss_and_grad(cfg, adj, rho0, vy0, W0, dts, 5, tgt)
    tr, tv = _taped_grad(cfg, W0, dts, tgt)
    err = torch.sqrt(((gr - tr) ** 2).sum() + ((gv - tv) ** 2).sum()) / torch.sqrt((tr ** 2).sum() + (tv ** 2).sum())
    assert float(err) < 1e-9, float(err)


def test_one_step_gradient_matches_finite_differences(cuda):
    """32 seeded directions, central differences with step 1e-8 on one step: 1e-6 relative."""
    cfg, _ = kh_setup(64, 32, "hlle", "rk2")
    adj = Adjoint(cfg)
    W0, Wt, dts, gen = _setup_rollout(cfg, 1, seed=13)
    with torch.no_grad():
        tgt = global_from_pack(cfg, adj.forward(pack_from_global(cfg, TR.prim_to_cons(Wt, cfg.gm1)), dts, 1))[0]
    rho0 = W0[0].clone().requires_grad_(True)
    vy0 = W0[2].clone().requires_grad_(True)
    _, gr, gv = _loss_and_grad(cfg, adj, rho0, vy0, W0, dts, 1, tgt)
    errs = _fd_rel(cfg, adj, W0, dts, 1, tgt, gr, gv, 1e-8, 32, gen)
    assert errs.max() < 1e-6, errs


def _taped_grad_checkpointed(cfg, W0, dts, tgt):
    """The taped restatement's gradient of a long rollout, one torch checkpoint per step (the
    graph of one step is rebuilt during the backward pass, so 200 steps of 512^2 fit)."""
    from torch.utils.checkpoint import checkpoint
    rho0 = W0[0].clone().requires_grad_(True)
    vy0 = W0[2].clone().requires_grad_(True)
    W = W0.clone()
    W[0] = rho0
    W[2] = vy0
    U = TR.prim_to_cons(W, cfg.gm1)
    for dt in dts:
        U = checkpoint(TR.step, U, dt, cfg.dx, cfg.gamma, cfg.recon, cfg.rsolver, cfg.integrator,
                       cfg.ndim, use_reentrant=False)
    loss = torch.sqrt(torch.sum((U[0] - tgt) ** 2))
    return torch.autograd.grad(loss, (rho0, vy0))


@pytest.mark.slow
def test_differentiable_kh_config_fd(cuda):
    """Differentiable KH 2D 512^2 (64 meshblocks of 64^2), PLM + HLLE, RK2, 200 steps with a
    checkpoint every 20, 32 seeded directions, central differences with step 1e-6.

    The adjoint's gradient equals the taped restatement's (torch.autograd through the same
    200 steps) to 1e-9, and on every direction the two directional derivatives agree to
    1e-9: the differences' disagreement with the gradient (median ~1e-3) is the same for
    both, so it belongs to the scheme's kinks (module docstring), not to the adjoint."""
    cfg, _ = kh_setup(512, 64, "hlle", "rk2")
    adj = Adjoint(cfg)
    W0, Wt, dts, gen = _setup_rollout(cfg, 200, seed=5)
    with torch.no_grad():
        tgt = global_from_pack(cfg, adj.forward(pack_from_global(cfg, TR.prim_to_cons(Wt, cfg.gm1)), dts, 20))[0]
    rho0 = W0[0].clone().requires_grad_(True)
    vy0 = W0[2].clone().requires_grad_(True)
    _, gr, gv = _loss_and_grad(cfg, adj, rho0, vy0, W0, dts, 20, tgt)
    tr, tv = _taped_grad_checkpointed(cfg, W0, dts, tgt)
    err = torch.sqrt(((gr - tr) ** 2).sum() + ((gv - tv) ** 2).sum()) / torch.sqrt((tr ** 2).sum() + (tv ** 2).sum())
    assert float(err) < 1e-9, float(err)
    errs, errs_taped = [], []
    h = 1e-6
    for _ in range(32):
        dr = torch.randn(gr.shape, dtype=torch.float64, device="cuda", generator=gen)
        dv = torch.randn(gv.shape, dtype=torch.float64, device="cuda", generator=gen)
        with torch.no_grad():
            lp = _loss_and_grad(cfg, adj, W0[0] + h * dr, W0[2] + h * dv, W0, dts, 20, tgt, False)
            lm = _loss_and_grad(cfg, adj, W0[0] - h * dr, W0[2] - h * dv, W0, dts, 20, tgt, False)
        fd = (lp - lm) / (2 * h)
        an = float((gr * dr).sum() + (gv * dv).sum())
        at = float((tr * dr).sum() + (tv * dv).sum())
        assert abs(an - at) <= 1e-9 * abs(at), (an, at)
        errs.append(abs(fd - an) / max(abs(fd), abs(an)))
        errs_taped.append(abs(fd - at) / max(abs(fd), abs(at)))
    errs, errs_taped = np.array(errs), np.array(errs_taped)
    print("differentiable KH config, FD relative errors: adjoint median %.2e max %.2e; taped "
          "median %.2e max %.2e" % (np.median(errs), errs.max(), np.median(errs_taped),
                                     errs_taped.max()))
    assert np.allclose(errs, errs_taped, rtol=1e-4, atol=1e-12)
    assert np.median(errs) < 1e-2 and errs.max() < 5e-2, errs


def _branches(cfg, W, dts):
    """The branch record of the taped restatement's rollout from primitive state W."""
    TR.BRANCHES = []
    try:
        with torch.no_grad():
            U = TR.prim_to_cons(W, cfg.gm1)
            for dt in dts:
                U = TR.step(U, dt, cfg.dx, cfg.gamma, cfg.recon, cfg.rsolver, cfg.integrator, cfg.ndim)
        return TR.BRANCHES
    finally:
        TR.BRANCHES = None


def test_ppm_hllc_gradient_matches_fd_where_no_branch_switches(cuda):
    """PPM + HLLC (2D KH, one 16^2 meshblock, 2 RK2 steps): on seeded directions whose
    central-difference pair u +- h d takes the same branch in every limiter and wave-speed
    decision of the rollout (the branch record of the taped restatement at both points), the
    adjoint's directional derivative agrees with the differences to 1e-6 relative.  The base
    state carries small cell-to-cell noise so that no decision is an exact tie (a smooth KH
    band is constant along x, and its zero second differences tie in PPM's min and sign
    tests); across a switched branch PPM's limiters jump and differences do not converge."""
    cfg, _ = kh_setup(16, 16, "hllc", "rk2", "ppm")
    adj = Adjoint(cfg)
    nsteps = 2
    W0, Wt, dts, _ = _setup_rollout(cfg, nsteps, seed=17)
    gen = torch.Generator().manual_seed(18)  # host generator: the same draws on every GPU
    noise = torch.randn(tuple(W0.shape), dtype=torch.float64, generator=gen) * 1e-3
    noise[3] = 0.0  # v_z stays exactly zero in 2D
    W0 = W0 + noise.cuda() * W0.abs().amax(dim=(1, 2, 3), keepdim=True)
    with torch.no_grad():
        tgt = global_from_pack(cfg, adj.forward(pack_from_global(cfg, TR.prim_to_cons(Wt, cfg.gm1)), dts, 1))[0]
    rho0 = W0[0].clone().requires_grad_(True)
    vy0 = W0[2].clone().requires_grad_(True)
    _, gr, gv = _loss_and_grad(cfg, adj, rho0, vy0, W0, dts, 1, tgt)
    h = 1e-8
    checked, errs = 0, []
    for _ in range(32):
        dr = torch.randn(tuple(gr.shape), dtype=torch.float64, generator=gen).cuda()
        dv = torch.randn(tuple(gv.shape), dtype=torch.float64, generator=gen).cuda()
        Wp, Wm = W0.clone(), W0.clone()
        Wp[0] += h * dr
        Wp[2] += h * dv
        Wm[0] -= h * dr
        Wm[2] -= h * dv
        bp, bm = _branches(cfg, Wp, dts), _branches(cfg, Wm, dts)
        if not all(torch.equal(a, b) for a, b in zip(bp, bm)):
            continue  # a branch switches between the two points
        with torch.no_grad():
            lp = _loss_and_grad(cfg, adj, Wp[0], Wp[2], W0, dts, 1, tgt, False)
            lm = _loss_and_grad(cfg, adj, Wm[0], Wm[2], W0, dts, 1, tgt, False)
        fd = (lp - lm) / (2 * h)
        an = float((gr * dr).sum() + (gv * dv).sum())
        errs.append(abs(fd - an) / max(abs(fd), abs(an)))
        checked += 1
    print("PPM+HLLC: %d of 32 directions without a switched branch; FD errors %s" % (
        checked, np.array2string(np.array(errs), precision=2)))
    assert checked >= 4
    assert max(errs) < 1e-6, errs


def test_checkpoint_spacing_does_not_change_gradient(cuda):
    cfg, cons = kh_setup(64, 32, "hllc", "rk2")
    adj = Adjoint(cfg)
    dts = [1.5e-3] * 12
    gen = torch.Generator(device="cuda").manual_seed(3)
    lam = pack_from_global(cfg, torch.randn((5, 1, 64, 64), dtype=torch.float64, device="cuda",
                                            generator=gen))
    outs = []
    for k in (1, 5, 12):
        uT = adj.forward(cons, dts, k)
        outs.append(adj.backward(lam))
    assert torch.equal(outs[0], outs[1]) and torch.equal(outs[1], outs[2])


def test_autotuned_forward_keeps_the_gradient(cuda):
    """Tuning the adjoint's forward (launch shape, sweep order, staging) changes nothing the
    taped reference can see."""
    cfg, u = kh_setup(64, 32, "hllc", "rk2", "ppm")
    adj = Adjoint(cfg)
    adj.autotune(u)
    dt = 2e-3
    G = global_from_pack(cfg, u).requires_grad_(True)
    ref_next = TR.step(G, dt, cfg.dx, cfg.gamma, cfg.recon, cfg.rsolver, cfg.integrator, cfg.ndim)
    gen = torch.Generator(device="cuda").manual_seed(3)
    lamG = torch.randn(ref_next.shape, dtype=torch.float64, device="cuda", generator=gen)
    (ref_vjp,) = torch.autograd.grad(ref_next, G, lamG)
    got_vjp = global_from_pack(cfg, adj.step_vjp(u, dt, pack_from_global(cfg, lamG)))
    assert float((got_vjp - ref_vjp).norm() / ref_vjp.norm()) < 1e-11
    adj.close()
