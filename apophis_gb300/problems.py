"""Synthetic initial conditions for the hydro path's workloads.

Each generator returns ``(cfg, cons)`` where ``cons`` is a pack
``(nblocks, 5, nk, nj, ni)`` of conserved variables with the interior set and
the ghost cells zero (the drivers fill ghosts).  They follow the conventions of
the reference's problem generators: src/pgen/sod.cpp:11-46, kh.cpp:71-119,
rt.cpp:18-104, blast.cpp:16-71, linear_wave.cpp:42-147 and 304-419.
Random perturbations come from numpy's PCG64 generator with a fixed seed.
"""
import dataclasses
import math

import numpy as np

from .mesh import DEFAULT_FLOOR, IDN, IEN, IM1, IM2, IM3, MeshConfig


def _alloc(cfg):
    return np.zeros(cfg.pack_shape(5), dtype=np.float64)


def _set_prim(cfg, cons, b, rho, vx, vy, vz, p):
    sk, sj, si = cfg.interior
    gm1 = cfg.gm1
    blk = cons[b]
    rho = np.broadcast_to(rho, blk[0][sk, sj, si].shape)
    blk[IDN][sk, sj, si] = rho
    blk[IM1][sk, sj, si] = rho * vx
    blk[IM2][sk, sj, si] = rho * vy
    blk[IM3][sk, sj, si] = rho * vz
    blk[IEN][sk, sj, si] = p / gm1 + 0.5 * rho * (vx * vx + vy * vy + vz * vz)


def sod(nx=256, x0=0.5, xmin=0.0, xmax=1.0, left=(1.0, 0.0, 1.0), right=(0.125, 0.0, 0.1),
        recon="plm", rsolver="hlle", integrator="rk2", cfl=0.4, gamma=1.4, ng=2, block_nx=None):
    """Sod shock tube, 1D, outflow boundaries (sod.cpp:11-46)."""
    cfg = MeshConfig(ndim=1, mesh_nx=(nx, 1, 1), block_nx=(block_nx or nx, 1, 1), ng=ng,
                     xmin=(xmin, -0.5, -0.5), xmax=(xmax, 0.5, 0.5),
                     bc=(("outflow", "outflow"), ("periodic", "periodic"), ("periodic", "periodic")),
                     recon=recon, rsolver=rsolver, integrator=integrator, cfl=cfl, gamma=gamma,
                     name="sod1d")
    cons = _alloc(cfg)
    for b in range(cfg.nblocks):
        x, _, _ = cfg.cell_centers(b)
        L = x < x0
        rho = np.where(L, left[0], right[0])
        u = np.where(L, left[1], right[1])
        p = np.where(L, left[2], right[2])
        _set_prim(cfg, cons, b, rho, u, 0.0, 0.0, p)
    return cfg, cons


def kh3d(n=256, block=64, ng=4, recon="ppm", rsolver="hllc", integrator="rk2", cfl=0.3,
         gamma=5.0 / 3.0, seed=0):
    """3D Kelvin-Helmholtz shear in the periodic unit box: rho 2 and vx +0.5 in the band
    |y-0.5|<0.25, rho 1 and vx -0.5 outside, p 2.5, vy = 0.01 sin(4 pi x) + U(-1e-3, 1e-3)."""
    cfg = MeshConfig(ndim=3, mesh_nx=(n, n, n), block_nx=(block, block, block), ng=ng,
                     recon=recon, rsolver=rsolver, integrator=integrator, cfl=cfl, gamma=gamma,
                     name="kh3d")
    cons = _alloc(cfg)
    rng = np.random.Generator(np.random.PCG64(seed))
    noise = rng.uniform(-1e-3, 1e-3, size=(n, n, n))
    bn = cfg.block_nx
    for b in range(cfg.nblocks):
        x, y, z = cfg.cell_centers(b)
        bi, bj, bk = cfg.block_index(b)
        band = np.abs(y - 0.5) < 0.25
        rho = np.where(band, 2.0, 1.0)
        vx = np.where(band, 0.5, -0.5)
        nz = noise[bk * bn[2]:(bk + 1) * bn[2], bj * bn[1]:(bj + 1) * bn[1],
                   bi * bn[0]:(bi + 1) * bn[0]]
        vy = 0.01 * np.sin(4.0 * math.pi * x) + nz
        _set_prim(cfg, cons, b, rho, vx, vy, 0.0, 2.5)
    return cfg, cons


def kh2d(n=512, block=64, ng=2, recon="plm", rsolver="hlle", integrator="rk2", cfl=0.3,
         gamma=5.0 / 3.0, seed=0, amp_noise=1e-3):
    """2D Kelvin-Helmholtz shear, periodic unit square, same profile as kh3d."""
    cfg = MeshConfig(ndim=2, mesh_nx=(n, n, 1), block_nx=(block, block, 1), ng=ng,
                     recon=recon, rsolver=rsolver, integrator=integrator, cfl=cfl, gamma=gamma,
                     name="kh2d")
    cons = _alloc(cfg)
    rng = np.random.Generator(np.random.PCG64(seed))
    noise = rng.uniform(-amp_noise, amp_noise, size=(n, n))
    bn = cfg.block_nx
    for b in range(cfg.nblocks):
        x, y, _ = cfg.cell_centers(b)
        bi, bj, _ = cfg.block_index(b)
        band = np.abs(y - 0.5) < 0.25
        rho = np.where(band, 2.0, 1.0)
        vx = np.where(band, 0.5, -0.5)
        nz = noise[bj * bn[1]:(bj + 1) * bn[1], bi * bn[0]:(bi + 1) * bn[0]][None]
        vy = 0.01 * np.sin(4.0 * math.pi * x) + nz
        _set_prim(cfg, cons, b, rho, vx, vy, 0.0, 2.5)
    return cfg, cons


def kh2d_smooth(n=512, block=64, ng=2, recon="plm", rsolver="hlle", integrator="rk2", cfl=0.3,
                gamma=5.0 / 3.0, width=0.05):
    """2D Kelvin-Helmholtz with resolved (tanh) shear layers at y = 0.25 and 0.75 and smooth
    perturbations in every field, periodic unit square (the profile family of kh.cpp's
    iprob=4).  No region is exactly flat, so the step is differentiable almost everywhere
    (a piecewise-constant state puts every flat cell on a kink of the PLM limiter)."""
    cfg = MeshConfig(ndim=2, mesh_nx=(n, n, 1), block_nx=(block, block, 1), ng=ng,
                     recon=recon, rsolver=rsolver, integrator=integrator, cfl=cfl, gamma=gamma,
                     name="kh2d_smooth")
    cons = _alloc(cfg)
    # layer positions and phases off the grid's symmetry lines: a profile mirrored about a
    # cell face gives pairs of equal cells, i.e. zero differences sitting on the limiter's kink
    y1, y2 = 0.25 + 0.0123, 0.75 + 0.0123
    for b in range(cfg.nblocks):
        x, y, _ = cfg.cell_centers(b)
        band = 0.5 * (np.tanh((y - y1) / width) - np.tanh((y - y2) / width))
        rho = 1.5 + 0.5 * band + 0.05 * np.sin(2.0 * math.pi * (x + 2.0 * y) + 0.37)
        vx = band - 0.5 + 0.02 * np.cos(2.0 * math.pi * (2.0 * x - y) + 1.13)
        vy = (0.01 * np.sin(4.0 * math.pi * x + 0.71) +
              0.005 * np.sin(2.0 * math.pi * (x + y) + 2.29))
        p = 2.5 + 0.05 * np.cos(2.0 * math.pi * (x - 3.0 * y) + 0.53)
        _set_prim(cfg, cons, b, rho, vx, vy, 0.0, p)
    return cfg, cons


def rt2d(nx=256, ny=768, block=(32, 32), ng=4, recon="ppm", rsolver="hllc", integrator="rk2",
         cfl=0.4, gamma=1.4, g=-0.1):
    """2D Rayleigh-Taylor on [0,0.5]x[0,1.5]: rho 2 above rho 1, hydrostatic pressure
    p = 1/gamma + g rho (y - 0.75), reflecting in y, periodic in x, constant gravity g in y
    (rt.cpp:18-104 with the interface at the domain centre)."""
    cfg = MeshConfig(ndim=2, mesh_nx=(nx, ny, 1), block_nx=(block[0], block[1], 1), ng=ng,
                     xmin=(0.0, 0.0, -0.5), xmax=(0.5, 1.5, 0.5),
                     bc=(("periodic", "periodic"), ("reflecting", "reflecting"),
                         ("periodic", "periodic")),
                     recon=recon, rsolver=rsolver, integrator=integrator, cfl=cfl, gamma=gamma,
                     gravity=(0.0, g, 0.0), name="rt2d")
    cons = _alloc(cfg)
    for b in range(cfg.nblocks):
        x, y, _ = cfg.cell_centers(b)
        xc, yc = x - 0.25, y - 0.75
        rho = np.where(yc < 0.0, 1.0, 2.0)
        vy = 0.01 * (1.0 + np.cos(4.0 * math.pi * xc)) * (1.0 + np.cos(3.0 * math.pi * yc)) / 4.0
        p = 1.0 / gamma + g * rho * yc
        _set_prim(cfg, cons, b, rho, 0.0, vy, 0.0, p)
    return cfg, cons


def blast2d(n=256, block=64, ng=4, r0=0.1, gamma=1.4, recon="ppm", rsolver="hllc",
            integrator="rk2", cfl=0.3, p_in=10.0, p_out=0.1):
    """2D blast wave in the periodic unit square: rho 1, p p_in inside r0 of the centre and
    p_out elsewhere (blast.cpp:16-71 without the pressure ramp)."""
    cfg = MeshConfig(ndim=2, mesh_nx=(n, n, 1), block_nx=(block, block, 1), ng=ng,
                     recon=recon, rsolver=rsolver, integrator=integrator, cfl=cfl, gamma=gamma,
                     name="blast2d")
    cons = _alloc(cfg)
    for b in range(cfg.nblocks):
        x, y, _ = cfg.cell_centers(b)
        r = np.sqrt((x - 0.5) ** 2 + (y - 0.5) ** 2)
        p = np.where(r < r0, p_in, p_out)
        _set_prim(cfg, cons, b, 1.0, 0.0, 0.0, 0.0, p)
    return cfg, cons


def rarefaction2d(n=48, block=16, ng=3, recon="ppm", rsolver="hllc", integrator="rk2", cfl=0.3,
                  gamma=1.4, v0=3.0, pfloor=0.1, dfloor=None):
    """Two-dimensional double rarefaction (Einfeldt's 1-2-3 problem, faster, turned 30 degrees
    off the x axis): rho 1, p 0.4, the two halves moving apart at v0 along the normal of the
    line through the centre, outflow boundaries.  The pressure between the two rarefactions
    falls below the raised pressure floor (the reference's hydro/pfloor) from the fourth step
    on, in the blocks along the line (5 of the 9 at the defaults) and in no other block."""
    cfg = MeshConfig(ndim=2, mesh_nx=(n, n, 1), block_nx=(block, block, 1), ng=ng,
                     recon=recon, rsolver=rsolver, integrator=integrator, cfl=cfl, gamma=gamma,
                     bc=(("outflow", "outflow"), ("outflow", "outflow"), ("periodic", "periodic")),
                     pfloor=pfloor, dfloor=dfloor if dfloor is not None else DEFAULT_FLOOR,
                     name="rarefaction2d")
    cons = _alloc(cfg)
    nx_, ny_ = math.cos(math.pi / 6), math.sin(math.pi / 6)
    for b in range(cfg.nblocks):
        x, y, _ = cfg.cell_centers(b)
        side = np.where((x - 0.5) * nx_ + (y - 0.5) * ny_ < 0.0, -1.0, 1.0)
        _set_prim(cfg, cons, b, 1.0, side * v0 * nx_, side * v0 * ny_, 0.0, 0.4)
    return cfg, cons


class LinearWave:
    """3D linear sound wave along the grid diagonal (linear_wave.cpp:42-147, 304-419):
    wave_flag 0, amplitude 1e-6, no background flow, domain [0,3]x[0,1.5]x[0,1.5]."""

    def __init__(self, res=16, recon="plm", rsolver="hllc", integrator="vl2", gamma=5.0 / 3.0,
                 amp=1e-6, cfl=0.3, ng=2, periods=2.0, block=None):
        nx = (2 * res, res, res)
        self.cfg = MeshConfig(ndim=3, mesh_nx=nx, block_nx=block or nx, ng=ng,
                              xmin=(0.0, 0.0, 0.0), xmax=(3.0, 1.5, 1.5), recon=recon,
                              rsolver=rsolver, integrator=integrator, cfl=cfl, gamma=gamma,
                              name="linear_wave3d")
        self.amp = amp
        gam = gamma
        gm1 = gam - 1.0
        x1s, x2s, x3s = 3.0, 1.5, 1.5
        ang_3 = math.atan(x1s / x2s)
        self.sin_a3, self.cos_a3 = math.sin(ang_3), math.cos(ang_3)
        ang_2 = math.atan(0.5 * (x1s * self.cos_a3 + x2s * self.sin_a3) / x3s)
        self.sin_a2, self.cos_a2 = math.sin(ang_2), math.cos(ang_2)
        x1 = x1s * self.cos_a2 * self.cos_a3
        x2 = x2s * self.cos_a2 * self.sin_a3
        x3 = x3s * self.sin_a2
        lam = x1
        if ang_3 != 0.0:
            lam = min(lam, x2)
        if ang_2 != 0.0:
            lam = min(lam, x3)
        self.k_par = 2.0 * math.pi / lam
        d0, u0 = 1.0, 0.0
        p0 = 1.0 / gam
        h0 = ((p0 / gm1 + 0.5 * d0 * (u0 * u0)) + p0) / d0
        a = math.sqrt(gm1 * max(h0 - 0.5 * u0 * u0, 1e-20))
        self.ev0 = u0 - a
        self.rem = (1.0, u0 - a, 0.0, 0.0, h0 - u0 * a)  # right eigenvector of wave 0
        self.d0, self.p0, self.gm1 = d0, p0, gm1
        self.tlim = lam / abs(self.ev0) * periods

    def solution(self):
        cfg = self.cfg
        cons = _alloc(cfg)
        sk, sj, si = cfg.interior
        for b in range(cfg.nblocks):
            X1, X2, X3 = cfg.cell_centers(b)
            x = self.cos_a2 * (X1 * self.cos_a3 + X2 * self.sin_a3) + X3 * self.sin_a2
            sn = np.sin(self.k_par * x)
            r = self.rem
            mx = self.amp * sn * r[1]
            my = self.amp * sn * r[2]
            mz = self.amp * sn * r[3]
            c = cons[b]
            c[IDN][sk, sj, si] = self.d0 + self.amp * sn * r[0]
            c[IM1][sk, sj, si] = mx * self.cos_a2 * self.cos_a3 - my * self.sin_a3 - mz * self.sin_a2 * self.cos_a3
            c[IM2][sk, sj, si] = mx * self.cos_a2 * self.sin_a3 + my * self.cos_a3 - mz * self.sin_a2 * self.sin_a3
            c[IM3][sk, sj, si] = mx * self.sin_a2 + mz * self.cos_a2
            c[IEN][sk, sj, si] = self.p0 / self.gm1 + self.amp * sn * r[4]
        return cons

    def rms_l1_error(self, cons):
        """RMS of the per-variable volume-weighted L1 errors (linear_wave.cpp:149-261)."""
        cfg = self.cfg
        ref = self.solution()
        sk, sj, si = cfg.interior
        dx = cfg.dx
        vol = dx[0] * dx[1] * dx[2]
        l1 = np.zeros(5)
        for b in range(cfg.nblocks):
            diff = np.abs(ref[b][:, sk, sj, si] - cons[b][:, sk, sj, si])
            l1 += diff.reshape(5, -1).sum(axis=1) * vol
        l1 /= 3.0 * 1.5 * 1.5
        return float(np.sqrt(np.sum(l1 * l1))), l1


def with_tracers(cfg, cons5, nscalars=2):
    """(cfg, cons) of any problem with passive scalars (dyes) added: scalar k is rho * s_k,
    s_0 a band in y (in x for 1D) and s_1 a smooth pattern in x, y, z, s_2 = s_0 ..."""
    tcfg = dataclasses.replace(cfg, nscalars=nscalars)
    cons = np.zeros(tcfg.pack_shape(tcfg.nvar))
    cons[:, :5] = cons5[:, :5]
    sk, sj, si = tcfg.interior
    for b in range(tcfg.nblocks):
        x, y, z = tcfg.cell_centers(b)
        rho = cons5[b, 0][sk, sj, si]
        q = y if tcfg.ndim >= 2 else x
        dyes = [0.5 * (np.tanh((q - 0.25) / 0.05) - np.tanh((q - 0.75) / 0.05)),
                0.5 + 0.25 * np.sin(2 * math.pi * x) * np.cos(2 * math.pi * y) * np.cos(2 * math.pi * z)]
        for k in range(nscalars):
            cons[b, 5 + k][sk, sj, si] = rho * dyes[k % 2]
    return tcfg, cons


def kh2d_tracers(n=64, block=32, ng=2, recon="plm", rsolver="hllc", integrator="rk2", cfl=0.3,
                 gamma=5.0 / 3.0, nscalars=2):
    """kh2d_smooth with passive scalars (dyes) advected by the flow: scalar k is
    rho * s_k with s_0 marking the central band and s_1 a smooth pattern in x and y."""
    cfg, cons5 = kh2d_smooth(n=n, block=block, ng=ng, recon=recon, rsolver=rsolver,
                             integrator=integrator, cfl=cfl, gamma=gamma)
    cfg, cons = with_tracers(cfg, cons5, nscalars)
    cfg.name = "kh2d_tracers"
    return cfg, cons
