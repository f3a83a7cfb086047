"""The C-ABI library: it builds, loads, exports every declared entry point, and rejects
bad arguments with a status code and a message (no GPU needed: argument checks run
before any CUDA call)."""
import ctypes
import os
import re

import pytest

from apophis_gb300 import _capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")


def declared_symbols():
    names = set()
    for fn in os.listdir(INCLUDE):
        if fn.endswith(".h"):
            src = open(os.path.join(INCLUDE, fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(aph_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    lib = _capi.load()
    names = declared_symbols()
    assert "aph_hydro_calculate_fluxes" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding knows every one of them
    known = set(_capi.SIGNATURES) | set(_capi.EXTRA_SIGNATURES)
    assert not [n for n in names if n not in known]


def _params(**kw):
    base = dict(ndim=2, nghost=3, nvar=5, recon=3, rsolver=3, gm1=0.4, dfloor=1e-18,
                pfloor=1e-18, cfl=0.3, exact=0)
    base.update(kw)
    return _capi.aph_hydro_params(*[base[f] for f, _ in _capi.aph_hydro_params._fields_])


def _block():
    b = _capi.aph_block()
    b.cons = 0x1000  # never dereferenced: creation fails in validation first
    b.nx[:] = [8, 8, 1]
    b.dx[:] = [0.1, 0.1, 1.0]
    return b


@pytest.mark.parametrize("kw,needle", [
    (dict(nghost=2, recon=3), "ghost"),
    (dict(recon=7), "reconstruction"),
    (dict(rsolver=9), "Riemann"),
    (dict(rsolver=1, recon=2), "none"),
    (dict(ndim=4), "ndim"),
    (dict(gm1=-1.0), "gm1"),
    (dict(nvar=3), "nvar"),
])
def test_pack_create_rejects_bad_params(kw, needle):
    lib = _capi.load()
    h = ctypes.c_void_p()
    blk = (_capi.aph_block * 1)(_block())
    st = lib.aph_pack_create(ctypes.byref(_params(**kw)), blk, 1, ctypes.byref(h))
    assert st == 1  # APH_ERR_INVALID
    assert needle in lib.aph_last_error().decode()
    assert not h.value


def test_pack_create_rejects_bad_blocks():
    lib = _capi.load()
    h = ctypes.c_void_p()
    b = _block()
    b.nx[2] = 4  # a third dimension in a 2D pack
    st = lib.aph_pack_create(ctypes.byref(_params()), (_capi.aph_block * 1)(b), 1, ctypes.byref(h))
    assert st == 1 and "nx3" in lib.aph_last_error().decode()
    b = _block()
    b.cons = None
    st = lib.aph_pack_create(ctypes.byref(_params()), (_capi.aph_block * 1)(b), 1, ctypes.byref(h))
    assert st == 1 and "cons" in lib.aph_last_error().decode()
    st = lib.aph_pack_create(None, (_capi.aph_block * 1)(_block()), 1, ctypes.byref(h))
    assert st == 1


def test_pack_create_rejects_flux_strides_too_small():
    """Caller-given flux layouts must hold each component's face array (a row of ni + 1
    faces along x1, nj + 1 rows along x2, planes of those rows)."""
    lib = _capi.load()
    h = ctypes.c_void_p()
    ni, nj = 8 + 6, 8 + 6  # nx + 2 nghost
    for d, strides in [(0, [ni * nj, ni * nj, ni]),            # x1 rows without the extra face
                       (1, [ni * nj, ni * nj, ni]),            # x2 planes without the extra row
                       (0, [1, (ni + 1) * nj, ni + 1])]:       # components overlapping
        b = _block()
        b.flux_stride[d][:] = strides
        st = lib.aph_pack_create(ctypes.byref(_params()), (_capi.aph_block * 1)(b), 1,
                                 ctypes.byref(h))
        assert st == 1 and "strides" in lib.aph_last_error().decode(), (d, strides)
        assert not h.value


def test_null_pack_calls_fail_cleanly():
    lib = _capi.load()
    assert lib.aph_hydro_cons_to_prim(None, None) == 1
    assert lib.aph_hydro_calculate_fluxes(None, 3, 3, None) == 1
    assert lib.aph_hydro_fill_ghosts(None, None) == 1
    d = ctypes.c_double()
    assert lib.aph_hydro_estimate_timestep(None, ctypes.byref(d), None) == 1
    assert lib.aph_pack_destroy(None) == 0


def test_null_stepper_calls_fail_cleanly():
    """Every stepper entry point checks its handle before any device work."""
    lib = _capi.load()
    d = ctypes.c_double()
    buf = (ctypes.c_double * 8)()
    assert lib.aph_stepper_step(None, 1, None) == 1
    assert lib.aph_stepper_status(None, ctypes.byref(d), ctypes.byref(d), None, None) == 1
    assert lib.aph_stepper_history(None, buf, None) == 1
    assert lib.aph_stepper_load_interiors(None, buf, None) == 1
    assert lib.aph_stepper_store_interiors(None, buf, None) == 1
    assert lib.aph_stepper_set_clock(None, 0.0, 0.0, 0, None) == 1
    assert lib.aph_stepper_destroy(None) == 0
    assert "NULL" in lib.aph_last_error().decode()


def test_stepper_rejects_bad_ensembles():
    """Validation runs before any device work, so it is checked without a GPU."""
    import ctypes
    from apophis_gb300 import ensemble, problems
    lib = _capi.load()
    cfgs = [problems.blast2d(n=32, block=16)[0], problems.blast2d(n=32, block=16)[0]]
    ens = ensemble.Ensemble(cfgs, [0.1, 0.1])
    blks = ens.blocks()
    nb = ens.nblocks
    blocks = (_capi.aph_block * nb)()
    for b, B in enumerate(blks):
        blocks[b].cons = 4096 * (b + 1)  # never dereferenced: validation fails first
        blocks[b].nx[:] = [B.nx[0], B.nx[1], 1]
        blocks[b].dx[:] = [B.dx[0], B.dx[1], 1.0]

    def make(edit_table=None, member=None, gm1=None):
        table = (_capi.aph_amr_block * nb)()
        for b, B in enumerate(blks):
            t = table[b]
            t.level = B.level
            t.origin[0], t.origin[1] = B.origin
            for f in range(4):
                t.face_kind[f] = B.face_kind[f]
                t.face_count[f] = len(B.face_nbr[f])
                for k, x in enumerate(B.face_nbr[f]):
                    t.face_nbr[f][k] = x
        if edit_table:
            edit_table(table)
        mem = (ctypes.c_int * nb)(*(member or ens.member_of))
        g = (ctypes.c_double * 2)(*(gm1 or [0.4, 0.5]))
        e = _capi.aph_ensemble(2, mem, g, None)
        desc = _capi.aph_stepper_desc()
        desc.params = _capi.aph_hydro_params(2, 2, 5, 3, 3, 0.4, 1e-10, 1e-10, 0.3, 0)
        desc.integrator = 2
        desc.nblocks = nb
        desc.blocks = ctypes.cast(blocks, ctypes.POINTER(_capi.aph_block))
        desc.nb[:] = [nb, 1, 1]
        desc.bc[:] = [0, 0, 0, 0, 0, 0]
        desc.amr = ctypes.cast(table, ctypes.POINTER(_capi.aph_amr_block))
        desc.ensemble = ctypes.pointer(e)
        h = ctypes.c_void_p()
        return lib.aph_stepper_create(ctypes.byref(desc), ctypes.byref(h)), (table, mem, g, e)

    def cross(t):  # block 0 of member 0 names block 4 (member 1) as its x- neighbour
        t[0].face_nbr[0][0] = 4

    for kw in (dict(edit_table=cross), dict(member=[0, 0, 0, 0, 1, 1, 1, 5]),
               dict(gm1=[0.4, -1.0])):
        st, _keep = make(**kw)
        assert st == 1, (kw, st, _capi.load().aph_last_error())  # APH_ERR_INVALID


def test_bad_ghost_width_and_floors_rejected():
    """Validation before any device work: PPM with 2 ghost cells (hydro.cpp:72-75)."""
    import ctypes
    lib = _capi.load()
    p = _capi.aph_hydro_params(2, 2, 5, 3, 3, 0.4, 1e-10, 1e-10, 0.3, 0)  # ppm, ng 2
    blk = (_capi.aph_block * 1)()
    blk[0].cons = 4096
    blk[0].nx[:] = [8, 8, 1]
    blk[0].dx[:] = [0.1, 0.1, 1.0]
    h = ctypes.c_void_p()
    assert lib.aph_pack_create(ctypes.byref(p), blk, 1, ctypes.byref(h)) == 1
