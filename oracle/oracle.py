"""ctypes loader for the CPU oracle (test infrastructure, not product code).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module: it is the checker the CUDA path is compared
against, and the CPU time that is reported beside it.  See ``hydro_oracle.cpp``
for the reference files each function restates.
"""
import ctypes
import os

import numpy as np

from . import build_oracle

_LIB = None

RECON = {"dc": 1, "plm": 2, "ppm": 3}
RSOLVER = {"none": 1, "hlle": 2, "hllc": 3, "lhllc": 4}
INTEGRATOR = {"rk1": 1, "rk2": 2, "rk3": 3, "vl2": 4}
BC = {"periodic": 0, "outflow": 1, "reflecting": 2}

_dp = ctypes.POINTER(ctypes.c_double)


def lib():
    global _LIB
    if _LIB is None:
        path = build_oracle.build()
        L = ctypes.CDLL(path)
        L.orc_estimate_dt.restype = ctypes.c_double
        L.orc_mesh_create.restype = ctypes.c_void_p
        L.orc_mesh_create.argtypes = [ctypes.POINTER(ctypes.c_int), _dp]
        L.orc_mesh_destroy.argtypes = [ctypes.c_void_p]
        L.orc_mesh_set_cons.argtypes = [ctypes.c_void_p, _dp]
        L.orc_mesh_get.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp]
        L.orc_mesh_run.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_double]
        L.orc_mesh_run.restype = ctypes.c_int
        L.orc_mesh_state.argtypes = [ctypes.c_void_p, _dp]
        L.orc_num_threads.restype = ctypes.c_int
        _LIB = L
    return _LIB


def _p(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


def set_num_threads(n):
    lib().orc_set_num_threads(int(n))


def num_threads():
    return lib().orc_num_threads()


# ---- single-block kernels ---------------------------------------------------------
def cons_to_prim(cons, prim, gamma, nx, ng, ndim, gm1, dfloor, pfloor):
    nvar = cons.shape[0]
    lib().orc_cons_to_prim(_p(cons), _p(prim), _p(gamma), nvar, nx[0], nx[1], nx[2], ng, ndim,
                           ctypes.c_double(gm1), ctypes.c_double(dfloor), ctypes.c_double(pfloor))


def calculate_fluxes(prim, gamma, flux, nx, ng, ndim, recon, rsolver):
    nvar = prim.shape[0]
    f = [_p(flux[d]) if d < ndim else None for d in range(3)]
    lib().orc_calculate_fluxes(_p(prim), _p(gamma), f[0], f[1], f[2], nvar, nx[0], nx[1], nx[2],
                               ng, ndim, RECON[recon], RSOLVER[rsolver])


def update(u0, u1, flux, nx, ng, ndim, dx, gam0, gam1, beta_dt):
    nvar = u0.shape[0]
    f = [_p(flux[d]) if d < ndim else None for d in range(3)]
    dxa = np.ascontiguousarray(dx, dtype=np.float64)
    lib().orc_update(_p(u0), _p(u1), f[0], f[1], f[2], nvar, nx[0], nx[1], nx[2], ng, ndim,
                     _p(dxa), ctypes.c_double(gam0), ctypes.c_double(gam1),
                     ctypes.c_double(beta_dt))


def estimate_dt(prim, cons, nx, ng, ndim, dx, cfl, gm1):
    nvar = cons.shape[0]
    dxa = np.ascontiguousarray(dx, dtype=np.float64)
    return lib().orc_estimate_dt(_p(prim), _p(cons), nvar, nx[0], nx[1], nx[2], ng, ndim,
                                 _p(dxa), ctypes.c_double(cfl), ctypes.c_double(gm1))


def apply_gravity(cons, prim, nx, ng, ndim, g, dt):
    nvar = cons.shape[0]
    ga = np.ascontiguousarray(g, dtype=np.float64)
    lib().orc_apply_gravity(_p(cons), _p(prim), nvar, nx[0], nx[1], nx[2], ng, ndim, _p(ga),
                            ctypes.c_double(dt))


def plm(a, b, c):
    l, r = ctypes.c_double(), ctypes.c_double()
    lib().orc_plm(ctypes.c_double(a), ctypes.c_double(b), ctypes.c_double(c), ctypes.byref(l),
                  ctypes.byref(r))
    return l.value, r.value


def ppm(a, b, c, d, e):
    l, r = ctypes.c_double(), ctypes.c_double()
    args = [ctypes.c_double(x) for x in (a, b, c, d, e)]
    lib().orc_ppm(*args, ctypes.byref(l), ctypes.byref(r))
    return l.value, r.value


def plm_many(q):
    """PLM of the stencils q (n, 3): (n, 2) array of (ql_{i+1}, qr_i)."""
    q = np.ascontiguousarray(q, dtype=np.float64)
    out = np.empty((q.shape[0], 2))
    lib().orc_plm_many(_p(q), _p(out), ctypes.c_long(q.shape[0]))
    return out


def ppm_many(q):
    """PPM of the stencils q (n, 5): (n, 2) array of (ql_{i+1}, qr_i)."""
    q = np.ascontiguousarray(q, dtype=np.float64)
    out = np.empty((q.shape[0], 2))
    lib().orc_ppm_many(_p(q), _p(out), ctypes.c_long(q.shape[0]))
    return out


def riemann(rsolver, wl, wr, gl, gr):
    out = np.zeros(5)
    arrs = [np.ascontiguousarray(x, dtype=np.float64) for x in (wl, wr, gl, gr)]
    lib().orc_riemann(RSOLVER[rsolver], *[_p(a) for a in arrs], _p(out))
    return out


# ---- uniform mesh driver ------------------------------------------------------------
class Mesh:
    """Uniform mesh of equal meshblocks driven in the reference's stage order."""

    def __init__(self, cfg):
        self.cfg = cfg
        nbx = cfg.blocks_per_dim
        bc = cfg.bc
        ints = [cfg.nvar, cfg.ndim, cfg.block_nx[0], cfg.block_nx[1], cfg.block_nx[2],
                nbx[0], nbx[1], nbx[2], cfg.ng, RECON[cfg.recon], RSOLVER[cfg.rsolver],
                INTEGRATOR[cfg.integrator],
                BC[bc[0][0]], BC[bc[0][1]], BC[bc[1][0]], BC[bc[1][1]], BC[bc[2][0]],
                BC[bc[2][1]], 1 if cfg.gravity is not None else 0]
        g = cfg.gravity if cfg.gravity is not None else (0.0, 0.0, 0.0)
        reals = [cfg.gm1, cfg.cfl, cfg.dfloor, cfg.pfloor, *cfg.dx, *g]
        self._ints = (ctypes.c_int * len(ints))(*ints)
        self._reals = (ctypes.c_double * len(reals))(*reals)
        self.h = lib().orc_mesh_create(self._ints, self._reals)
        self.shape = cfg.pack_shape(cfg.nvar)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_mesh_destroy(self.h)
            self.h = None

    def set_cons(self, cons):
        c = np.ascontiguousarray(cons, dtype=np.float64)
        assert c.shape == self.shape, (c.shape, self.shape)
        lib().orc_mesh_set_cons(self.h, _p(c))

    def get(self, what="cons"):
        idx = {"cons": 0, "prim": 1, "gamma": 2, "u1": 3, "flux1": 4, "flux2": 5, "flux3": 6}[what]
        shape = self.shape if what != "gamma" else self.shape[:1] + (2,) + self.shape[2:]
        out = np.empty(shape, dtype=np.float64)
        lib().orc_mesh_get(self.h, idx, _p(out))
        return out

    def run(self, nsteps=1 << 30, tlim=1e300, fixed_dt=0.0):
        return lib().orc_mesh_run(self.h, int(nsteps), ctypes.c_double(tlim),
                                  ctypes.c_double(fixed_dt))

    def state(self):
        out = np.zeros(3)
        lib().orc_mesh_state(self.h, _p(out))
        return {"time": out[0], "dt": out[1], "ncycle": int(out[2])}


class AmrMesh:
    """Statically refined 2D mesh (apophis_gb300.amr.AmrConfig) driven by the oracle."""

    def __init__(self, cfg):
        self.cfg = cfg
        bc = cfg.bc
        ints = [cfg.nblocks, cfg.ng, RECON[cfg.recon], RSOLVER[cfg.rsolver],
                INTEGRATOR[cfg.integrator], BC[bc[0][0]], BC[bc[0][1]], BC[bc[1][0]],
                BC[bc[1][1]], 1 if cfg.gravity is not None else 0, cfg.nvar]
        blk = []
        bdx = []
        for B in cfg.blocks:
            row = [B.level, B.origin[0], B.origin[1], B.nx[0], B.nx[1]]
            row += list(B.face_kind) + [len(n) for n in B.face_nbr]
            for n in B.face_nbr:
                row += list(n) + [0] * (4 - len(n))
            blk += row
            bdx += [B.dx[0], B.dx[1], 1.0]
        g = cfg.gravity if cfg.gravity is not None else (0.0, 0.0, 0.0)
        reals = [cfg.gm1, cfg.cfl, cfg.dfloor, cfg.pfloor, *g]
        L = lib()
        L.orc_amr_create.restype = ctypes.c_void_p
        L.orc_amr_create.argtypes = [ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int), _dp, _dp]
        L.orc_amr_destroy.argtypes = [ctypes.c_void_p]
        L.orc_amr_set_cons.argtypes = [ctypes.c_void_p, _dp]
        L.orc_amr_get.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp]
        L.orc_amr_run.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_double]
        L.orc_amr_run.restype = ctypes.c_int
        L.orc_amr_state.argtypes = [ctypes.c_void_p, _dp]
        self._keep = [(ctypes.c_int * len(ints))(*ints), (ctypes.c_int * len(blk))(*blk),
                      (ctypes.c_double * len(reals))(*reals), (ctypes.c_double * len(bdx))(*bdx)]
        self.h = L.orc_amr_create(*self._keep)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_amr_destroy(self.h)
            self.h = None

    def set_cons(self, cons):
        c = np.ascontiguousarray(cons, dtype=np.float64)
        assert c.size == self.cfg.flat_size()
        lib().orc_amr_set_cons(self.h, _p(c))

    def get(self, what="cons"):
        out = np.empty(self.cfg.flat_size())
        lib().orc_amr_get(self.h, 0 if what == "cons" else 1, _p(out))
        return out

    def plant_no_correction(self):
        """Tests only: make the oracle skip the coarse-fine flux correction."""
        lib().orc_amr_plant_no_correction(ctypes.c_void_p(self.h))

    def run(self, nsteps=1 << 30, tlim=1e300, fixed_dt=0.0):
        return lib().orc_amr_run(self.h, int(nsteps), ctypes.c_double(tlim), ctypes.c_double(fixed_dt))

    def state(self):
        out = np.zeros(3)
        lib().orc_amr_state(self.h, _p(out))
        return {"time": out[0], "dt": out[1], "ncycle": int(out[2])}


def history(cfg, cons):
    """GlobalQuantHst<Sum, IDN / IEN> (src/hydro/hydro.cpp:754-771): the sums over interior
    cells of cons * CellVolume, for a uniform pack (nblocks, nvar, nk, nj, ni)."""
    sk, sj, si = cfg.interior
    vol = float(np.prod(cfg.dx))
    inner = np.asarray(cons)[:, :, sk, sj, si]
    return {"total_mass": float(inner[:, 0].sum() * vol),
            "total_energy": float(inner[:, 4].sum() * vol)}
