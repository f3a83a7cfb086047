"""ctypes binding of include/aph_hydro.h (libaph_hydro.so)."""
import ctypes
import os

from . import _build

_LIB = None

APH_OK = 0
APH_STAGE_GHOSTS_GIVEN = 1
STATUS_NAMES = {0: "APH_OK", 1: "APH_ERR_INVALID", 2: "APH_ERR_UNSUPPORTED", 3: "APH_ERR_CUDA",
                4: "APH_ERR_TIMEOUT", 5: "APH_ERR_STATE"}
RECON = {"dc": 1, "plm": 2, "ppm": 3}
RSOLVER = {"none": 1, "hlle": 2, "hllc": 3, "lhllc": 4}
INTEGRATOR = {"rk1": 1, "rk2": 2, "rk3": 3, "vl2": 4}
BC = {"periodic": 0, "outflow": 1, "reflecting": 2}

_dp = ctypes.POINTER(ctypes.c_double)


class aph_block(ctypes.Structure):
    _fields_ = [("cons", ctypes.c_void_p), ("prim", ctypes.c_void_p), ("gamma", ctypes.c_void_p),
                ("u1", ctypes.c_void_p), ("flux", ctypes.c_void_p * 3),
                ("nx", ctypes.c_int * 3), ("dx", ctypes.c_double * 3),
                ("flux_stride", (ctypes.c_longlong * 3) * 3), ("eos_lambda", ctypes.c_void_p)]


class aph_hydro_params(ctypes.Structure):
    _fields_ = [("ndim", ctypes.c_int), ("nghost", ctypes.c_int), ("nvar", ctypes.c_int),
                ("recon", ctypes.c_int), ("rsolver", ctypes.c_int), ("gm1", ctypes.c_double),
                ("dfloor", ctypes.c_double), ("pfloor", ctypes.c_double),
                ("cfl", ctypes.c_double), ("exact", ctypes.c_int)]


class aph_amr_block(ctypes.Structure):
    _fields_ = [("level", ctypes.c_int), ("origin", ctypes.c_int * 2),
                ("face_kind", ctypes.c_int * 4), ("face_count", ctypes.c_int * 4),
                ("face_nbr", (ctypes.c_int * 4) * 4)]


class aph_ensemble(ctypes.Structure):
    _fields_ = [("nmembers", ctypes.c_int), ("member", ctypes.POINTER(ctypes.c_int)),
                ("gm1", ctypes.POINTER(ctypes.c_double)),
                ("tlim", ctypes.POINTER(ctypes.c_double))]


class aph_stepper_desc(ctypes.Structure):
    _fields_ = [("params", aph_hydro_params), ("integrator", ctypes.c_int),
                ("nblocks", ctypes.c_int), ("blocks", ctypes.POINTER(aph_block)),
                ("nb", ctypes.c_int * 3), ("bc", ctypes.c_int * 6),
                ("use_gravity", ctypes.c_int), ("gravity", ctypes.c_double * 3),
                ("tlim", ctypes.c_double), ("fixed_dt", ctypes.c_double),
                ("amr", ctypes.POINTER(aph_amr_block)),
                ("ensemble", ctypes.POINTER(aph_ensemble))]


class aph_stepper_config(ctypes.Structure):
    _fields_ = [("threads", ctypes.c_int), ("ctas_per_sm", ctypes.c_int),
                ("lines", ctypes.c_int * 3), ("order", ctypes.c_int * 3),
                ("schedule", ctypes.c_int), ("use_graph", ctypes.c_int),
                ("reg_cap", ctypes.c_int), ("tma", ctypes.c_int)]

    def to_dict(self):
        return {"threads": self.threads, "ctas_per_sm": self.ctas_per_sm,
                "lines": list(self.lines), "order": list(self.order),
                "schedule": self.schedule, "use_graph": self.use_graph,
                "reg_cap": self.reg_cap, "tma": self.tma}

    @classmethod
    def from_dict(cls, d):
        c = cls()
        c.threads = d["threads"]
        c.ctas_per_sm = d.get("ctas_per_sm", 0)
        c.lines[:] = d["lines"]
        c.order[:] = d["order"]
        c.schedule = d["schedule"]
        c.use_graph = d.get("use_graph", 1)
        c.reg_cap = d.get("reg_cap", 0)
        c.tma = d.get("tma", 0)
        return c


class AphError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), msg))
        self.status = status


# (name, argtypes) of every entry point; also the list the ABI tests check.
SIGNATURES = {
    "aph_last_error": ([], ctypes.c_char_p),
    "aph_version": ([], ctypes.c_int),
    "aph_pack_create": ([ctypes.POINTER(aph_hydro_params), ctypes.POINTER(aph_block), ctypes.c_int,
                         ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "aph_pack_set_topology": ([ctypes.c_void_p, ctypes.POINTER(ctypes.c_int),
                               ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
    "aph_pack_set_amr": ([ctypes.c_void_p, ctypes.POINTER(aph_amr_block),
                          ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
    "aph_amr_check": ([ctypes.POINTER(aph_amr_block), ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                       ctypes.c_int], ctypes.c_int),
    "aph_pack_partition": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                            ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "aph_pack_destroy": ([ctypes.c_void_p], ctypes.c_int),
    "aph_hydro_cons_to_prim": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "aph_hydro_calculate_fluxes": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p],
                                   ctypes.c_int),
    "aph_hydro_update_with_flux_divergence": ([ctypes.c_void_p, ctypes.c_double, ctypes.c_double,
                                               ctypes.c_double, ctypes.c_void_p], ctypes.c_int),
    "aph_hydro_update_with_flux_divergence_dev": ([ctypes.c_void_p, ctypes.c_double,
                                                   ctypes.c_double, ctypes.c_double,
                                                   ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "aph_hydro_estimate_timestep": ([ctypes.c_void_p, _dp, ctypes.c_void_p], ctypes.c_int),
    "aph_hydro_estimate_timestep_async": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
                                          ctypes.c_int),
    "aph_hydro_apply_gravity": ([ctypes.c_void_p, _dp, ctypes.c_double, ctypes.c_void_p],
                                ctypes.c_int),
    "aph_hydro_fill_ghosts": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "aph_hydro_estimate_timestep_noalloc": ([ctypes.c_void_p, ctypes.c_void_p,
                                             ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                                             ctypes.c_int, _dp, ctypes.c_double, ctypes.c_double,
                                             ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "aph_stepper_create": ([ctypes.POINTER(aph_stepper_desc), ctypes.POINTER(ctypes.c_void_p)],
                           ctypes.c_int),
    "aph_stepper_destroy": ([ctypes.c_void_p], ctypes.c_int),
    "aph_stepper_step": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p], ctypes.c_int),
    "aph_stepper_status": ([ctypes.c_void_p, _dp, _dp, ctypes.POINTER(ctypes.c_int),
                            ctypes.c_void_p], ctypes.c_int),
    "aph_hydro_history": ([ctypes.c_void_p, _dp, ctypes.c_void_p], ctypes.c_int),
    "aph_stepper_history": ([ctypes.c_void_p, _dp, ctypes.c_void_p], ctypes.c_int),
    "aph_stepper_load_interiors": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "aph_stepper_store_interiors": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "aph_stepper_set_clock": ([ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                               ctypes.c_void_p], ctypes.c_int),
    "aph_diag_barrier_timeout": ([ctypes.c_double, ctypes.c_void_p], ctypes.c_int),
    "aph_stepper_stage": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p],
                          ctypes.c_int),
    "aph_stepper_local_dt": ([ctypes.c_void_p, _dp, ctypes.c_void_p], ctypes.c_int),
    "aph_stepper_end_step": ([ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p], ctypes.c_int),
    "aph_diag_exact_ops": ([ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong,
                            ctypes.c_void_p], ctypes.c_int),
    "aph_diag_exact_ops2": ([ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                             ctypes.c_longlong, ctypes.c_void_p], ctypes.c_int),
    "aph_stepper_member_status": ([ctypes.c_void_p, _dp, _dp, ctypes.POINTER(ctypes.c_int),
                                   ctypes.c_void_p], ctypes.c_int),
    "aph_stepper_get_config": ([ctypes.c_void_p, ctypes.POINTER(aph_stepper_config)],
                               ctypes.c_int),
    "aph_stepper_set_config": ([ctypes.c_void_p, ctypes.POINTER(aph_stepper_config)],
                               ctypes.c_int),
    "aph_stepper_profile": ([ctypes.c_void_p, ctypes.c_int, _dp, ctypes.c_void_p], ctypes.c_int),
    "aph_stepper_autotune": ([ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(aph_stepper_config),
                              _dp], ctypes.c_int),
    "aph_adjoint_create": ([ctypes.POINTER(aph_stepper_desc), ctypes.POINTER(ctypes.c_void_p)],
                           ctypes.c_int),
    "aph_adjoint_destroy": ([ctypes.c_void_p], ctypes.c_int),
    "aph_adjoint_step": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p,
                          ctypes.c_void_p], ctypes.c_int),
    "aph_adjoint_step_vjp": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p,
                              ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "aph_adjoint_forward": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, _dp, ctypes.c_int,
                             ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "aph_adjoint_forward_members": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, _dp,
                                     ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "aph_adjoint_autotune": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "aph_adjoint_backward": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
                             ctypes.c_int),
}
EXTRA_SIGNATURES = {}


def lib_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load the shared library (building it first when it is missing)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if build_if_missing:
        path = _build.build()
    if not os.path.exists(path):
        raise RuntimeError("libaph_hydro.so is not built; run __graft_entry__.build()")
    L = ctypes.CDLL(path)
    for name, (argtypes, restype) in {**SIGNATURES, **EXTRA_SIGNATURES}.items():
        if not hasattr(L, name):
            continue
        fn = getattr(L, name)
        fn.argtypes = argtypes
        fn.restype = restype
    _LIB = L
    return L


def check(status):
    if status != APH_OK:
        msg = load().aph_last_error()
        raise AphError(status, msg.decode() if msg else "")
    return status


def call(name, *args):
    return check(getattr(load(), name)(*args))
