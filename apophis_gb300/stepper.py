"""The batched path: a whole pack advanced by full RK steps (aph_stepper_* in
include/aph_hydro.h).

Each RK stage is one persistent launch over every meshblock; dt and time stay on the
device; a step is captured once as a CUDA graph and replayed.  ``Stepper`` owns the
state tensor ``cons`` (nblocks, nvar, nk, nj, ni); the C library owns the rest.
Launch configurations found by ``autotune`` are cached in a JSON file keyed by the
workload and the GPU.
"""
import ctypes
import json
import os

import numpy as np
import torch

from . import _capi
from .hydro import make_params, require_cuda, stream_handle
from .mesh import MeshConfig

TUNE_CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "autotune.json")


class Stepper:
    def __init__(self, cfg: MeshConfig, cons0=None, exact=True, tlim=None, fixed_dt=0.0,
                 cons=None, dx=None):
        require_cuda()
        _capi.load()
        self.cfg = cfg
        self.exact = exact
        if cons is None:
            cons = torch.zeros(cfg.pack_shape(cfg.nvar), dtype=torch.float64, device="cuda")
            cons.copy_(torch.as_tensor(np.ascontiguousarray(cons0)))
        self.cons = cons
        blocks = (_capi.aph_block * cfg.nblocks)()
        dx = cfg.dx if dx is None else dx  # explicit widths: a rank's share of a larger mesh
        for b in range(cfg.nblocks):
            blocks[b].cons = self.cons[b].data_ptr()
            for d in range(3):
                blocks[b].nx[d] = cfg.block_nx[d]
                blocks[b].dx[d] = dx[d]
        self._blocks = blocks
        desc = _capi.aph_stepper_desc()
        desc.params = make_params(cfg, exact, cfg.nvar)
        desc.integrator = _capi.INTEGRATOR[cfg.integrator]
        desc.nblocks = cfg.nblocks
        desc.blocks = ctypes.cast(blocks, ctypes.POINTER(_capi.aph_block))
        desc.nb[:] = list(cfg.blocks_per_dim)
        desc.bc[:] = [_capi.BC[cfg.bc[d][s]] for d in range(3) for s in range(2)]
        desc.use_gravity = 1 if cfg.gravity is not None else 0
        desc.gravity[:] = list(cfg.gravity) if cfg.gravity is not None else [0.0, 0.0, 0.0]
        desc.tlim = tlim if tlim is not None else 0.0
        desc.fixed_dt = fixed_dt
        self.h = ctypes.c_void_p()
        _capi.call("aph_stepper_create", ctypes.byref(desc), ctypes.byref(self.h))

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            _capi.load().aph_stepper_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, nsteps=1, stream=None):
        _capi.call("aph_stepper_step", self.h, int(nsteps), stream_handle(stream))

    def status(self, stream=None):
        t, dt, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
        _capi.call("aph_stepper_status", self.h, ctypes.byref(t), ctypes.byref(dt),
                   ctypes.byref(n), stream_handle(stream))
        return {"time": t.value, "dt": dt.value, "ncycle": n.value}

    def save(self, base):
        """Checkpoint: the state as an output dump (output.write_dump) with the clock."""
        from . import output
        st = self.status()
        output.write_dump(base, self.cfg, self.state(), st["time"], st["ncycle"])
        import json
        meta = json.load(open(base + ".json"))
        meta["NextDt"] = st["dt"]
        meta["Exact"] = int(self.exact)
        with open(base + ".json", "w") as f:
            json.dump(meta, f, indent=1)

    @classmethod
    def restore(cls, base, cfg: MeshConfig, exact=None, tlim=None):
        """Resume from save(): the dump's interiors (ghosts are refilled by the first stage)
        and its clock."""
        from . import output
        d = output.Dump(base)
        cons = np.zeros(cfg.pack_shape(cfg.nvar))
        sk, sj, si = cfg.interior
        cons[:, :, sk, sj, si] = d.Get("cons", flatten=False)
        st = cls(cfg, cons, exact=bool(d.meta.get("Exact", 0)) if exact is None else exact, tlim=tlim)
        _capi.call("aph_stepper_set_clock", st.h, float(d.Time), float(d.meta["NextDt"]),
                   int(d.NCycle), stream_handle())
        return st

    def interior_shape(self):
        """Shape of the packed interiors: (nblocks, nvar, nx3, nx2, nx1)."""
        c = self.cfg
        return (c.nblocks, c.nvar, c.block_nx[2], c.block_nx[1], c.block_nx[0])

    def interior_values(self):
        """Length of the packed interiors (every block's nvar x interior cells)."""
        return self.cfg.nvar * self.cfg.zones()

    def _packed(self, a):
        n = self.interior_values()
        if isinstance(a, torch.Tensor):
            if a.dtype != torch.float64 or not a.is_contiguous() or a.numel() != n:
                raise ValueError("packed interiors: a contiguous float64 tensor of %d values" % n)
            return a.data_ptr()
        if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"] or a.size != n:
            raise ValueError("packed interiors: a C-contiguous float64 array of %d values" % n)
        return a.ctypes.data

    def load_interiors(self, src, stream=None):
        """Replace the state's interiors with the packed array src (interior_shape; device,
        pinned host or other host memory; asynchronous on the stream)."""
        _capi.call("aph_stepper_load_interiors", self.h, self._packed(src), stream_handle(stream))

    def store_interiors(self, dst, stream=None):
        """Write the state's interiors into the packed array dst (interior_shape)."""
        _capi.call("aph_stepper_store_interiors", self.h, self._packed(dst), stream_handle(stream))

    def history(self, stream=None):
        """GlobalQuantHst of the state: {"total_mass", "total_energy"}."""
        out = (ctypes.c_double * 2)()
        _capi.call("aph_stepper_history", self.h, out, stream_handle(stream))
        return {"total_mass": out[0], "total_energy": out[1]}

    def run(self, nsteps=1 << 30, tlim=float("inf"), check_every=16):
        """Step until nsteps or tlim (checking the device clock every check_every steps)."""
        done = 0
        while done < nsteps:
            k = min(check_every, nsteps - done)
            self.step(k)
            done += k
            if tlim != float("inf") and self.status()["time"] >= tlim:
                break
        return self.status()

    def profile(self, nsteps=2, stream=None):
        """Mean duration (ms) of each stage launch over nsteps steps (advances the state)."""
        from .hydro import STAGES
        ns = len(STAGES[self.cfg.integrator])
        out = (ctypes.c_double * ns)()
        _capi.call("aph_stepper_profile", self.h, int(nsteps), out, stream_handle(stream))
        return list(out)

    @property
    def config(self):
        c = _capi.aph_stepper_config()
        _capi.call("aph_stepper_get_config", self.h, ctypes.byref(c))
        return c.to_dict()

    def set_config(self, d):
        c = _capi.aph_stepper_config.from_dict(d)
        _capi.call("aph_stepper_set_config", self.h, ctypes.byref(c))

    def tune_key(self):
        cfg = self.cfg
        dev = torch.cuda.get_device_name()
        return "%s|%s|nd%d|mesh%s|blk%s|ng%d|nvar%d|%s|%s|%s|exact%d" % (
            dev, cfg.name, cfg.ndim, "x".join(map(str, cfg.mesh_nx)),
            "x".join(map(str, cfg.block_nx)), cfg.ng, cfg.nvar, cfg.recon, cfg.rsolver,
            cfg.integrator, int(self.exact))

    def autotune(self, trial_steps=2, cache=TUNE_CACHE, use_cache=True):
        """Pick the fastest launch configuration (cached per workload and GPU)."""
        key = self.tune_key()
        db = {}
        if cache and os.path.exists(cache):
            try:
                db = json.load(open(cache))
            except (OSError, ValueError):
                db = {}
        if use_cache and key in db:
            try:
                self.set_config(db[key]["config"])
                return db[key]
            except _capi.AphError:
                pass
        best = _capi.aph_stepper_config()
        ms = ctypes.c_double()
        _capi.call("aph_stepper_autotune", self.h, int(trial_steps), ctypes.byref(best),
                   ctypes.byref(ms))
        rec = {"config": best.to_dict(), "ms_per_step": ms.value}
        if cache:
            db[key] = rec
            os.makedirs(os.path.dirname(cache), exist_ok=True)
            tmp = cache + ".tmp%d" % os.getpid()
            with open(tmp, "w") as f:
                json.dump(db, f, indent=1)
            os.replace(tmp, cache)
        return rec

    def state(self):
        torch.cuda.synchronize()
        return self.cons.cpu().numpy()


def smoke(cfg, cons, want):
    """One batched RK step of (cfg, cons) in exact mode must equal the oracle's `want`."""
    st = Stepper(cfg, cons, exact=True)
    st.step(1)
    got = st.state()
    sk, sj, si = cfg.interior
    assert np.array_equal(got[:, :, sk, sj, si], want[:, :, sk, sj, si]), \
        "batched exact step differs from the oracle"
    st.close()
