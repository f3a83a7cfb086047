"""Output dumps of a uniform pack and a reader with the part of Parthenon's phdf interface the
reference's analyses use (``Get(var)`` and ``GetVolumeLocations()``, as called at
tst/regression/test_suites/riemann_hydro/riemann_hydro.py:134-137), so those analyses can be
re-run on this library's output.

Format: ``<base>.json`` (metadata: time, cycle, mesh and block geometry, variable names and
the byte layout) and ``<base>.bin`` (raw little-endian float64: for each variable set in the
order listed, the interior cells of every block as (nblocks, nvar, nk, nj, ni)).  Both are
plain enough to read from any language.
"""
import json

import numpy as np

from .mesh import MeshConfig

CONS_NAMES = ["density", "momentum_x", "momentum_y", "momentum_z", "total_energy"]
PRIM_NAMES = ["density", "velocity_x", "velocity_y", "velocity_z", "pressure"]


def write_dump(base, cfg: MeshConfig, cons, time=0.0, ncycle=0, prim=None):
    """cons (and optionally prim): (nblocks, nvar, nk, nj, ni) with ghosts, numpy or torch;
    components past the fifth are passive scalars."""
    def interior(a):
        a = a.detach().cpu().numpy() if hasattr(a, "detach") else np.asarray(a)
        sk, sj, si = cfg.interior
        return np.ascontiguousarray(a[:, :, sk, sj, si], dtype="<f8")

    def names(base, a):
        return base + ["scalar_%d" % k for k in range(a.shape[1] - len(base))]

    c = interior(cons)
    sets = [("cons", c, names(CONS_NAMES, c))]
    if prim is not None:
        w = interior(prim)
        sets.append(("prim", w, names(PRIM_NAMES, w)))
    meta = {
        "format": "apophis_gb300 dump 1",
        "Time": float(time), "NCycle": int(ncycle),
        "NumDimensions": cfg.ndim, "NumMeshBlocks": cfg.nblocks,
        "MeshBlockSize": list(cfg.block_nx), "RootGridSize": list(cfg.mesh_nx),
        "RootGridDomain": [cfg.xmin[0], cfg.xmax[0], cfg.xmin[1], cfg.xmax[1], cfg.xmin[2], cfg.xmax[2]],
        "BlocksPerDim": list(cfg.blocks_per_dim),
        "Gamma": cfg.gamma,
        "Variables": [{"name": n, "components": names, "shape": list(a.shape), "dtype": "<f8"}
                      for n, a, names in sets],
    }
    with open(base + ".bin", "wb") as f:
        for _, a, _ in sets:
            f.write(a.tobytes())
    with open(base + ".json", "w") as f:
        json.dump(meta, f, indent=1)


class Dump:
    """Reader: ``Get(name)`` -> (nblocks, nk*nj*ni, nvar) like phdf's ``Get`` with flattened cells
    (``flatten=False``: (nblocks, nvar, nk, nj, ni)); ``GetVolumeLocations()`` -> per-block
    (z, y, x) cell-centre coordinates, flattened alike."""

    def __init__(self, base):
        if base.endswith(".json") or base.endswith(".bin"):
            base = base[:-5] if base.endswith(".json") else base[:-4]
        self.meta = json.load(open(base + ".json"))
        raw = np.fromfile(base + ".bin", dtype="<f8")
        self.vars = {}
        off = 0
        for v in self.meta["Variables"]:
            n = int(np.prod(v["shape"]))
            self.vars[v["name"]] = raw[off:off + n].reshape(v["shape"])
            off += n
        self.Time = self.meta["Time"]
        self.NCycle = self.meta["NCycle"]

    def Get(self, name, flatten=True):
        a = self.vars[name]
        if not flatten:
            return a
        nb, nv = a.shape[:2]
        return np.moveaxis(a.reshape(nb, nv, -1), 1, 2)

    def GetVolumeLocations(self, flatten=True):
        m = self.meta
        bs = m["MeshBlockSize"]
        nbd = m["BlocksPerDim"]
        dom = m["RootGridDomain"]
        dx = [(dom[2 * d + 1] - dom[2 * d]) / m["RootGridSize"][d] for d in range(3)]
        zs, ys, xs = [], [], []
        for b in range(m["NumMeshBlocks"]):
            loc = (b % nbd[0], (b // nbd[0]) % nbd[1], b // (nbd[0] * nbd[1]))
            c = [dom[2 * d] + (loc[d] * bs[d] + np.arange(bs[d]) + 0.5) * dx[d] for d in range(3)]
            z, y, x = np.meshgrid(c[2], c[1], c[0], indexing="ij")
            zs.append(z), ys.append(y), xs.append(x)
        out = [np.array(a) for a in (zs, ys, xs)]
        if flatten:
            out = [a.reshape(a.shape[0], -1) for a in out]
        return tuple(out)
