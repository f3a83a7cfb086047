"""ctypes binding of include/aph_hydro.h (libaph_hydro.so)."""
import ctypes
import os

from . import _build

_LIB = None

APH_OK = 0
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
                ("nx", ctypes.c_int * 3), ("dx", ctypes.c_double * 3)]


class aph_hydro_params(ctypes.Structure):
    _fields_ = [("ndim", ctypes.c_int), ("nghost", ctypes.c_int), ("nvar", ctypes.c_int),
                ("recon", ctypes.c_int), ("rsolver", ctypes.c_int), ("gm1", ctypes.c_double),
                ("dfloor", ctypes.c_double), ("pfloor", ctypes.c_double),
                ("cfl", ctypes.c_double), ("exact", ctypes.c_int)]


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
