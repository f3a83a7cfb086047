"""PyTorch FP64 restatement of the fixed-dt hydro step on a periodic global grid, for the
taped reference gradient of the adjoint tests (test infrastructure only).

It follows the same formulas as the CUDA fast path: ConsToPrim, PPM (ppm_simple.hpp:32-161),
PLM (plm_simple.hpp:15-32) or donor cell, HLLE (hydro_hlle.hpp:28-133) or HLLC (hydro_hllc.hpp:14-146) with the
c-limited sound speed written as sqrt(C^2 gamma p / (p (1 + 1/gm1) + rho C^2)), the flux
divergence and the low-storage RK stages.  torch.autograd differentiates it.
"""
import torch

C2 = 2.99792458e10 ** 2
TINY = 1.0e-20

# Branch record: while BRANCHES is a list, every limiter and wave-speed decision (the boolean
# masks of the piecewise definitions) is appended to it, so that two evaluations can be checked
# for taking the same branches everywhere (no kink between them).
BRANCHES = None


def _rec(*masks):
    if BRANCHES is not None:
        BRANCHES.extend(m.detach().clone() for m in masks)
STAGES = {
    "rk1": [(0.0, 1.0, 1.0)],
    "rk2": [(0.0, 1.0, 1.0), (0.5, 0.5, 0.5)],
    "rk3": [(0.0, 1.0, 1.0), (0.25, 0.75, 0.25), (2.0 / 3.0, 1.0 / 3.0, 2.0 / 3.0)],
    "vl2": [(0.0, 1.0, 0.5), (0.0, 1.0, 1.0)],
}


def c2p(U, gm1):
    rho = U[0]
    v = U[1:4] / rho
    ek = 0.5 * (U[1] ** 2 + U[2] ** 2 + U[3] ** 2) / rho
    p = gm1 * (U[4] - ek)
    return torch.cat([rho[None], v, p[None]], 0)


def prim_to_cons(W, gm1):
    rho = W[0]
    m = rho * W[1:4]
    E = W[4] / gm1 + 0.5 * rho * (W[1] ** 2 + W[2] ** 2 + W[3] ** 2)
    return torch.cat([rho[None], m, E[None]], 0)


def _ppm(q, axis, G):
    """PPM face states (the face/cell split of the CUDA path, with its limiter branches)."""
    n = q.shape[axis] - 2 * G
    sl = lambda a, b: q.narrow(axis, a + G, b - a)  # cells a..b-1
    C2 = 1.25
    Q4 = sl(-2, n + 2)                        # cells -2..n+1
    qm, qp = sl(-3, n + 1), sl(-1, n + 3)
    dd = 0.5 * (qp - Q4) + 0.5 * (Q4 - qm)
    d2 = (qm + qp) - 2.0 * Q4
    nf = n + 3                                # faces -1..n+1: between cells f-1 and f
    qm1, q0 = Q4.narrow(axis, 0, nf), Q4.narrow(axis, 1, nf)
    ddm1, dd0 = dd.narrow(axis, 0, nf), dd.narrow(axis, 1, nf)
    d2m1, d20 = d2.narrow(axis, 0, nf), d2.narrow(axis, 1, nf)
    avg = 0.5 * (qm1 + q0)
    dph = avg + (ddm1 - dd0) / 6.0
    qa_tmp, qb_tmp = dph - qm1, q0 - dph
    qa = 3.0 * (qm1 + q0 - 2.0 * dph)
    sa = qa < 0
    match = (sa == (d2m1 < 0)) & (sa == (d20 < 0))
    m = C2 * torch.where(d20.abs() < d2m1.abs(), d20.abs(), d2m1.abs())
    qd_mag_is_qa = qa.abs() < m
    qd = torch.where(qd_mag_is_qa, qa, torch.where(sa, -m, m))
    qd = torch.where(match, qd, torch.zeros_like(qd))
    _rec(sa, d2m1 < 0, d20 < 0, d20.abs() < d2m1.abs(), qd_mag_is_qa, qa_tmp * qb_tmp < 0)
    dph = torch.where(qa_tmp * qb_tmp < 0, avg - qd / 6.0, dph)
    nc = n + 2                                # cells -1..n
    lo, hi = dph.narrow(axis, 0, nc), dph.narrow(axis, 1, nc)
    qim2, qim1, qi, qip1, qip2 = (sl(-3, n - 1), sl(-2, n), sl(-1, n + 1), sl(0, n + 2),
                                  sl(1, n + 3))
    e2m1, e20, e2p1 = d2.narrow(axis, 0, nc), d2.narrow(axis, 1, nc), d2.narrow(axis, 2, nc)
    d2qf = 6.0 * (lo + hi - 2.0 * qi)
    dqm, dqp = qi - lo, hi - qi
    ext = ~(dqm * dqp > 0) | ~((qip1 - qi) * (qi - qim1) > 0)
    sd = d2qf < 0
    smatch = (sd == (e2m1 < 0)) & (sd == (e20 < 0)) & (sd == (e2p1 < 0))
    mm = torch.minimum(torch.minimum(e2m1.abs(), e20.abs()), e2p1.abs()) * C2
    qe_mag = torch.where(d2qf.abs() < mm, d2qf.abs(), mm)
    qe = torch.where(smatch, torch.where(sd, -qe_mag, qe_mag), torch.zeros_like(qe_mag))
    mx = torch.stack([qim2.abs(), qim1.abs(), qi.abs(), qip1.abs(), qip2.abs()]).amax(0)
    big = d2qf.abs() > 1e-12 * mx
    rho = torch.where(big, qe / torch.where(big, d2qf, torch.ones_like(d2qf)), torch.zeros_like(d2qf))
    app = rho <= 1.0 - 1e-12
    qr_e = torch.where(app, qi - rho * dqm, lo)
    ql_e = torch.where(app, qi + rho * dqp, hi)
    qr_m = torch.where(dqm.abs() >= 2.0 * dqp.abs(), qi - 2.0 * dqp, lo)
    ql_m = torch.where(dqp.abs() >= 2.0 * dqm.abs(), qi + 2.0 * dqm, hi)
    _rec(dqm * dqp > 0, (qip1 - qi) * (qi - qim1) > 0, sd, e2m1 < 0, e20 < 0, e2p1 < 0,
         e20.abs() < e2m1.abs(), e2p1.abs() < torch.minimum(e2m1.abs(), e20.abs()),
         d2qf.abs() < mm, big, app, dqm < 0, dqp < 0, dqm.abs() >= 2.0 * dqp.abs(),
         dqp.abs() >= 2.0 * dqm.abs())
    ql = torch.where(ext, ql_e, ql_m)
    qr = torch.where(ext, qr_e, qr_m)
    return ql.narrow(axis, 0, n + 1), qr.narrow(axis, 1, n + 1)


def _recon(q, recon, axis, G=2):
    """q padded by G cells along axis; returns left/right face states for faces 0..n: left
    from cell f-1, right from cell f."""
    if recon == "ppm":
        return _ppm(q, axis, G)
    n = q.shape[axis] - 2 * G
    sl = lambda a, b: q.narrow(axis, a + G, b - a)  # cells a..b-1
    if recon == "dc":
        return sl(-1, n), sl(0, n + 1)
    qm, q0, qp = sl(-2, n), sl(-1, n + 1), sl(0, n + 2)  # around cells -1..n
    dql = q0 - qm
    dqr = qp - q0
    dq2 = dql * dqr
    pos = dq2 > 0
    _rec(pos)
    den = torch.where(pos, dql + dqr, torch.ones_like(dql))
    dqm = torch.where(pos, dq2 / den, torch.zeros_like(dql))
    qlp = q0 + dqm  # left state of face c+1, c = -1..n
    qr = q0 - dqm   # right state of face c
    L = qlp.narrow(axis, 0, n + 1)   # faces 0..n from cells -1..n-1
    R = qr.narrow(axis, 1, n + 1)    # faces 0..n from cells 0..n
    return L, R


def _sound(rho, p, gamma, igm1):
    return torch.sqrt(C2 * gamma * p / (p * (1.0 + igm1) + rho * C2))


def hlle(wl, wr, gamma):
    igm1 = 1.0 / (gamma - 1.0)
    k = (gamma + 1.0) / (2.0 * gamma) ** 0.5
    rl, ul, vl, zl, pl = wl
    rr, ur, vr, zr, pr = wr
    cl, cr = _sound(rl, pl, gamma, igm1), _sound(rr, pr, gamma, igm1)
    el = pl * igm1 + 0.5 * rl * (ul ** 2 + vl ** 2 + zl ** 2)
    er = pr * igm1 + 0.5 * rr * (ur ** 2 + vr ** 2 + zr ** 2)
    rhoa = 0.5 * (rl + rr)
    ca = 0.5 * (cl + cr)
    pmid = 0.5 * (pl + pr + (ul - ur) * rhoa * ca)
    ql = torch.where(pmid > pl, 1.0 + k * (pmid / pl - 1.0), torch.ones_like(pl))
    qr = torch.where(pmid > pr, 1.0 + k * (pmid / pr - 1.0), torch.ones_like(pr))
    al = ul - cl * ql
    ar = ur + cr * qr
    _rec(pmid > pl, pmid > pr, ar > 0, al < 0)
    bp = torch.where(ar > 0, ar, torch.zeros_like(ar))
    bm = torch.where(al < 0, al, torch.zeros_like(al))
    vxl, vxr = ul - bm, ur - bp
    fl = [rl * vxl, rl * ul * vxl + pl, rl * vl * vxl, rl * zl * vxl, el * vxl + pl * ul]
    fr = [rr * vxr, rr * ur * vxr + pr, rr * vr * vxr, rr * zr * vxr, er * vxr + pr * ur]
    has = (bp != 0) | (bm != 0)
    den = torch.where(has, bp - bm, torch.ones_like(bp))
    tmp = torch.where(has, 0.5 * (bp + bm) / den, torch.zeros_like(bp))
    return [0.5 * (a + b) + (a - b) * tmp for a, b in zip(fl, fr)]


def hllc(wl, wr, gamma):
    igm1 = 1.0 / (gamma - 1.0)
    k = (gamma + 1.0) / (2.0 * gamma)
    rl, ul, vl, zl, pl = wl
    rr, ur, vr, zr, pr = wr
    cl, cr = _sound(rl, pl, gamma, igm1), _sound(rr, pr, gamma, igm1)
    el = pl * igm1 + 0.5 * rl * (ul ** 2 + vl ** 2 + zl ** 2)
    er = pr * igm1 + 0.5 * rr * (ur ** 2 + vr ** 2 + zr ** 2)
    rhoa = 0.5 * (rl + rr)
    ca = 0.5 * (cl + cr)
    pstar = 0.5 * (pl + pr) - 0.5 * (ur - ul) * rhoa * ca
    bl, br = pstar > pl, pstar > pr
    ql = torch.where(bl, torch.sqrt(torch.where(bl, 1.0 + k * (pstar / pl - 1.0), torch.ones_like(pl))),
                     torch.ones_like(pl))
    qr = torch.where(br, torch.sqrt(torch.where(br, 1.0 + k * (pstar / pr - 1.0), torch.ones_like(pr))),
                     torch.ones_like(pr))
    sl = ul - cl * ql
    sr = ur + cr * qr
    bp = torch.where(sr > 0, sr, torch.full_like(sr, TINY))
    bm = torch.where(sl < 0, sl, torch.full_like(sl, -TINY))
    vxl, vxr = ul - sl, ur - sr
    tl = pl + vxl * rl * ul
    tr = pr + vxr * rr * ur
    ml = rl * vxl
    mr = -(rr * vxr)
    sstar = (tl - tr) / (ml + mr)
    cp = (ml * tr + mr * tl) / (ml + mr)
    _rec(bl, br, sr > 0, sl < 0, cp > 0, sstar >= 0)
    cp = torch.where(cp > 0, cp, torch.zeros_like(cp))
    wxl, wxr = ul - bm, ur - bp
    fl = [rl * wxl, rl * ul * wxl + pl, rl * vl * wxl, rl * zl * wxl, el * wxl + pl * ul]
    fr = [rr * wxr, rr * ur * wxr + pr, rr * vr * wxr, rr * zr * wxr, er * wxr + pr * ur]
    sp = sstar >= 0
    dpos = torch.where(sp, sstar - bm, torch.ones_like(sstar))
    dneg = torch.where(sp, torch.ones_like(sstar), bp - sstar)
    cl_ = torch.where(sp, sstar / dpos, torch.zeros_like(sstar))
    cr_ = torch.where(sp, torch.zeros_like(sstar), -sstar / dneg)
    ustar = torch.where(sp, -bm / dpos, bp / dneg)
    out = [cl_ * a + cr_ * b for a, b in zip(fl, fr)]
    out[1] = out[1] + ustar * cp
    out[4] = out[4] + ustar * cp * sstar
    return out


def rhs(U, dx, gamma, recon, rsolver, ndim):
    """R(U) = -div F on a periodic global grid U (5, NZ, NY, NX)."""
    gm1 = gamma - 1.0
    axes = [3, 2, 1][:ndim]  # x, y, z axes of (var, z, y, x)
    G = 3 if recon == "ppm" else 2
    pad = U
    for ax in axes:
        n = pad.shape[ax]
        pad = torch.cat([pad.narrow(ax, n - G, G), pad, pad.narrow(ax, 0, G)], ax)
    W = c2p(pad, gm1)
    out = torch.zeros_like(U)
    solve = hlle if rsolver == "hlle" else hllc
    for d, ax in enumerate(axes):
        # crop the transverse padding: keep interior along the other axes
        Wd = W
        for od, oax in enumerate(axes):
            if oax != ax:
                Wd = Wd.narrow(oax, G, Wd.shape[oax] - 2 * G)
        L, R = _recon(Wd, recon, ax, G)
        ivx = 1 + d
        ivy = 1 + (d + 1) % 3
        ivz = 1 + (d + 2) % 3
        perm = [0, ivx, ivy, ivz, 4]
        wl = [L[v] for v in perm]
        wr = [R[v] for v in perm]
        f = solve(wl, wr, gamma)
        F = [None] * 5
        for k, v in enumerate(perm):
            F[v] = f[k]
        F = torch.stack(F, 0)
        n = F.shape[ax] - 1
        out = out - (F.narrow(ax, 1, n) - F.narrow(ax, 0, n)) / dx[d]
    return out


def step(U, dt, dx, gamma, recon, rsolver, integrator, ndim):
    Un = U
    u = U
    for s, (g0, g1, b) in enumerate(STAGES[integrator]):
        rc = "dc" if (integrator == "vl2" and s == 0) else recon
        u = g0 * u + g1 * Un + b * dt * rhs(u, dx, gamma, rc, rsolver, ndim)
    return u
