"""The oracle against the reference's own code (CPU).

oracle/_ref/libref_pin.so is the reference's reconstruction headers (src/recon/plm_simple.hpp,
ppm_simple.hpp, dc_simple.hpp) and Riemann solvers (src/hydro/rsolvers/hydro_{none,hlle,hllc,
lhllc}.hpp) compiled from their sources where they lie (oracle/build_ref.py, against the
stand-ins of oracle/ref_shim/ for the Parthenon / Kokkos names they use).  Every function the
oracle restates from those files must give the same bits as the reference's, on a million
random and edge stencils each, on Riemann states across every wave-speed branch and all
three directions, and on whole x1 flux rows of 1D blocks (Reconstruct<recon, X1DIR> +
Riemann::Solve + the passive-scalar upwinding of hydro.cpp:580-616).

The library is built where the reference checkout exists (this container); elsewhere these
tests are skipped.
"""
import ctypes
import zlib

import numpy as np
import pytest

from oracle import build_ref
from oracle import oracle as O

_dp = ctypes.POINTER(ctypes.c_double)


@pytest.fixture(scope="module")
def ref():
    path = build_ref.build()
    if path is None:
        pytest.skip("the reference checkout is not available: oracle/_ref not built")
    L = ctypes.CDLL(path)
    L.ref_plm.argtypes = [_dp, _dp, ctypes.c_long]
    L.ref_ppm.argtypes = [_dp, _dp, ctypes.c_long]
    L.ref_riemann.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, _dp, _dp, ctypes.c_int]
    L.ref_riemann.restype = ctypes.c_int
    L.ref_x1_fluxes.argtypes = [ctypes.c_int] * 5 + [_dp, _dp, _dp]
    L.ref_x1_fluxes.restype = ctypes.c_int
    return L


def _p(a):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


def _same(a, b, what):
    """Bitwise equality (NaNs compared as NaNs); reports the first difference."""
    a, b = np.asarray(a), np.asarray(b)
    same = (a.view(np.int64) == b.view(np.int64)) | (np.isnan(a) & np.isnan(b))
    if not same.all():
        idx = np.argwhere(~same)[0]
        raise AssertionError("%s: %d of %d differ; first at %s: oracle %r reference %r" % (
            what, (~same).sum(), same.size, tuple(idx), a[tuple(idx)], b[tuple(idx)]))


def _stencils(rng, n, width):
    """n stencils of the given width mixing the regimes the limiters branch on."""
    k = n // 8
    parts = [
        rng.standard_normal((k, width)),                                    # rough
        np.cumsum(rng.standard_normal((k, width)) * 1e-3, axis=1) + 1.0,    # smooth
        np.sort(rng.uniform(0.1, 10.0, (k, width)), axis=1),                # monotone
        np.repeat(rng.uniform(-1, 1, (k, 1)), width, axis=1),               # constant
        # constant plus round-off noise (the PPM roundoff guards, ppm_simple.hpp:132, 145)
        1.0 + rng.integers(-3, 4, (k, width)) * np.finfo(float).eps,
        # steps: a discontinuity at a random position (extremum and overshoot branches)
        np.where(np.arange(width)[None, :] < rng.integers(0, width + 1, (k, 1)),
                 rng.uniform(0.5, 2.0, (k, 1)), rng.uniform(0.05, 0.5, (k, 1))),
        # near-ties: values drawn from a few levels (face value equal to the cell average)
        rng.integers(-2, 3, (k, width)) * 0.25,
    ]
    rest = n - k * len(parts)
    # magnitudes from tiny to huge, with signed zeros
    scale = 10.0 ** rng.integers(-300, 300, (rest, 1))
    e = rng.standard_normal((rest, width)) * scale
    e[rng.random((rest, width)) < 0.1] = 0.0
    e[rng.random((rest, width)) < 0.05] = -0.0
    parts.append(e)
    return np.ascontiguousarray(np.concatenate(parts))


def test_plm_bit_identical(ref):
    q = _stencils(np.random.Generator(np.random.PCG64(1)), 1_000_000, 3)
    want = np.empty((q.shape[0], 2))
    ref.ref_plm(_p(q), _p(want), q.shape[0])
    _same(O.plm_many(q), want, "PLM")


def test_ppm_bit_identical(ref):
    q = _stencils(np.random.Generator(np.random.PCG64(2)), 1_000_000, 5)
    want = np.empty((q.shape[0], 2))
    ref.ref_ppm(_p(q), _p(want), q.shape[0])
    _same(O.ppm_many(q), want, "PPM")


def _states(rng, n, gamma):
    """Primitive (rho, v1, v2, v3, p) left/right states: smooth pairs, shocks, rarefactions,
    near-vacuum and identical states; adiabatic indices with round-off noise."""
    wl = np.empty((5, n))
    wr = np.empty((5, n))
    rho = rng.uniform(0.1, 3.0, (2, n))
    p = 10.0 ** rng.uniform(-3, 2, (2, n))
    v = rng.standard_normal((2, 3, n)) * rng.choice([0.0, 0.01, 1.0, 5.0], size=(2, 1, n))
    wl[0], wr[0] = rho
    wl[4], wr[4] = p
    wl[1:4], wr[1:4] = v
    same = rng.random(n) < 0.1
    wr[:, same] = wl[:, same]
    gl = np.empty((2, n))
    gr = np.empty((2, n))
    eps = np.finfo(float).eps
    for g in (gl, gr):
        g[0] = gamma * (1.0 + rng.integers(-4, 5, n) * eps)
        g[1] = gamma * (1.0 + rng.integers(-4, 5, n) * eps)
    return wl, wr, gl, gr


@pytest.mark.parametrize("rsolver", ["none", "hlle", "hllc", "lhllc"])
@pytest.mark.parametrize("ivx", [1, 2, 3])
def test_riemann_bit_identical(ref, rsolver, ivx):
    rng = np.random.Generator(np.random.PCG64(10 * ivx + O.RSOLVER[rsolver]))
    n = 50_000
    for gamma in (1.4, 5.0 / 3.0):
        wl, wr, gl, gr = _states(rng, n, gamma)
        want = np.zeros((5, n))
        assert ref.ref_riemann(O.RSOLVER[rsolver], ivx, _p(wl), _p(wr), _p(gl), _p(gr), _p(want),
                               n) == 0
        # the oracle's solver takes (rho, v_normal, v_t1, v_t2, p) and returns fluxes in that
        # order; the reference rotates by ivy = IV1 + ((ivx - IV1) + 1) % 3 (hydro_hllc.hpp:20-21)
        ivy = 1 + ((ivx - 1) + 1) % 3
        ivz = 1 + ((ivx - 1) + 2) % 3
        order = [0, ivx, ivy, ivz, 4]
        got = np.empty((5, n))
        for f in range(n):
            flx = O.riemann(rsolver, wl[order, f], wr[order, f], gl[:, f], gr[:, f])
            got[order, f] = flx
        _same(got, want, "%s ivx=%d gamma=%g" % (rsolver, ivx, gamma))


@pytest.mark.parametrize("recon,ng", [("dc", 2), ("plm", 2), ("ppm", 3), ("ppm", 4)])
@pytest.mark.parametrize("rsolver", ["hlle", "hllc", "lhllc"])
@pytest.mark.parametrize("nvar", [5, 7])
def test_x1_flux_rows_bit_identical(ref, recon, rsolver, nvar, ng):
    """Whole rows: Reconstruct<recon, X1DIR> of prim and gamma, Riemann::Solve over the
    faces of the interior and the mass-flux upwinding of passive scalars, against the
    oracle's calculate_fluxes of a 1D block."""
    seed = zlib.crc32(("%s %s %d %d" % (recon, rsolver, nvar, ng)).encode())
    rng = np.random.Generator(np.random.PCG64(seed))
    nx = 64
    ni = nx + 2 * ng
    for trial in range(20):
        prim = np.empty((nvar, ni))
        x = np.arange(ni)
        jump = rng.integers(0, ni)
        prim[0] = np.where(x < jump, 1.0, 0.125) + 0.01 * rng.standard_normal(ni) * (trial % 2)
        prim[1] = rng.standard_normal(ni) * 0.5
        prim[2] = rng.standard_normal(ni) * 0.1 * (trial % 3 != 0)
        prim[3] = 0.0 if trial % 4 == 0 else rng.standard_normal(ni) * 0.1
        prim[4] = np.where(x < jump, 1.0, 0.1) * (1.0 + 0.1 * rng.random(ni))
        for n in range(5, nvar):
            prim[n] = rng.random(ni)
        gamma = 1.4 * (1.0 + rng.integers(-3, 4, (2, ni)) * np.finfo(float).eps)
        want = np.zeros((nvar, ni))
        assert ref.ref_x1_fluxes(O.RECON[recon], O.RSOLVER[rsolver], nvar, nx, ng, _p(prim),
                                 _p(np.ascontiguousarray(gamma)), _p(want)) == 0
        flux = [np.zeros((nvar, 1, 1, ni))]
        O.calculate_fluxes(prim.reshape(nvar, 1, 1, ni).copy(),
                           np.ascontiguousarray(gamma.reshape(2, 1, 1, ni)), flux,
                           (nx, 1, 1), ng, 1, recon, rsolver)
        got = flux[0].reshape(nvar, ni)
        faces = slice(ng, ng + nx + 1)
        _same(got[:, faces], want[:, faces], "%s+%s nvar %d trial %d" % (recon, rsolver, nvar, trial))
