"""Shared helpers of the parity tests: small workloads and the tolerance rule.

Tolerance for the fast arithmetic mode, per cell and per variable n:
    |gpu - oracle| <= RTOL * max(|oracle|, scale_n),   RTOL = 1e-12,
where scale_n is the largest |value| of variable n over the compared region, and for the
three momentum components the largest |value| of any momentum component (momentum is
one vector: a component that is born from cancellation, such as the z momentum of a
flow that starts planar, carries the rounding of the O(|m|) terms it came from).  Fluxes
are compared the same way with one scale for the whole flux vector (vector=True): a flux
component that cancels to zero in the reference, such as the mass flux of a fluid at rest
under a pressure jump, carries the rounding of the O(|F|) terms of the solver.  The exact
mode must match bit for bit.

The fast mode is held to this tolerance for one step.  Over several steps it can leave
it: the reference's PPM limiter switches branches discontinuously (for instance between
its extremum and overshoot formulas when a face value equals the cell average), so a
one-ulp difference in a degenerate stencil can change a face value by the size of the
local jump.  Multi-step bit stability is what the exact mode is for.
"""
import numpy as np

from apophis_gb300 import problems

RTOL = 1e-12


def assert_parity(gpu, ref, exact, rtol=RTOL, what="", vector=False):
    gpu = np.asarray(gpu)
    ref = np.asarray(ref)
    assert gpu.shape == ref.shape, (gpu.shape, ref.shape)
    if exact:
        same = (gpu == ref) | (np.isnan(gpu) & np.isnan(ref))
        if not same.all():
            idx = np.argwhere(~same)[0]
            raise AssertionError("%s: %d cells differ bitwise; first at %s: gpu %r ref %r" % (
                what, (~same).sum(), tuple(idx), gpu[tuple(idx)], ref[tuple(idx)]))
        return
    # per-variable scale along axis 1 (nvar) of (nblocks, nvar, ...) arrays
    nv = ref.shape[1]
    mom = np.max(np.abs(ref[:, 1:4])) if ref.size and nv >= 4 else 0.0
    whole = np.max(np.abs(ref[:, :5])) if ref.size else 0.0
    for n in range(nv):
        r = ref[:, n]
        g = gpu[:, n]
        scale = np.max(np.abs(r)) if r.size else 0.0
        if 1 <= n <= 3:
            scale = max(scale, mom)
        if vector and n < 5:
            scale = max(scale, whole)
        tol = rtol * np.maximum(np.abs(r), scale)
        bad = np.abs(g - r) > tol
        if bad.any():
            idx = np.argwhere(bad)[0]
            raise AssertionError("%s var %d: %d cells off; first at %s: gpu %r ref %r (tol %r)" % (
                what, n, bad.sum(), tuple(idx), g[tuple(idx)], r[tuple(idx)], tol[tuple(idx)]))


def small_workloads():
    """(name, cfg, cons) of small cases covering 1D/2D/3D, every solver and boundary."""
    out = []
    cfg, cons = problems.sod(nx=64, recon="plm", rsolver="hlle", integrator="rk2", ng=2)
    out.append(("sod_plm_hlle", cfg, cons))
    cfg, cons = problems.sod(nx=64, recon="ppm", rsolver="hllc", integrator="rk2", ng=3,
                             block_nx=16)
    out.append(("sod_ppm_hllc_4blocks", cfg, cons))
    cfg, cons = problems.kh2d(n=32, block=16, ng=3, recon="ppm", rsolver="hllc")
    out.append(("kh2d_ppm_hllc", cfg, cons))
    cfg, cons = problems.kh2d(n=32, block=16, ng=2, recon="plm", rsolver="hlle")
    out.append(("kh2d_plm_hlle", cfg, cons))
    cfg, cons = problems.kh2d(n=32, block=32, ng=2, recon="plm", rsolver="lhllc")
    out.append(("kh2d_plm_lhllc", cfg, cons))
    cfg, cons = problems.kh3d(n=16, block=8, ng=4, recon="ppm", rsolver="hllc")
    out.append(("kh3d_ppm_hllc", cfg, cons))
    cfg, cons = problems.rt2d(nx=16, ny=48, block=(8, 16), ng=4)
    out.append(("rt2d_ppm_hllc_gravity", cfg, cons))
    cfg, cons = problems.blast2d(n=32, block=16, ng=3, recon="ppm", rsolver="hlle")
    out.append(("blast2d_ppm_hlle", cfg, cons))
    return out


def interior_faces(cfg, d):
    """Slices (k, j, i) of the faces of direction d that the update reads."""
    sk, sj, si = cfg.interior
    sl = [sk, sj, si]
    ax = 2 - d
    s = sl[ax]
    sl[ax] = slice(s.start, s.stop + 1)
    return tuple(sl)


def l1_rel(gpu, ref, n=0):
    """Mean |gpu - ref| of variable n over the mean |ref|."""
    return float(np.mean(np.abs(gpu[:, n] - ref[:, n])) / np.mean(np.abs(ref[:, n])))
