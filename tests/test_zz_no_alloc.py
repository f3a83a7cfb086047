"""The allocation-free timestep estimate, called through the C ABI (needs a GPU).

aph_hydro_estimate_timestep_noalloc serves callers that may not allocate device memory
(a pool allocator has taken it up front, and an allocation mid-step would synchronise).  Two calls in a row must
agree with the regular aph_hydro_estimate_timestep on the same meshblock, within the
fast-mode tolerance of the parity tests, and blocks above the stated maximum are refused.
This file is collected last so that a run that stops at the first failure has already run
every other test; it also passes on its own in a fresh process (its first call sets up the
device scratch).
"""
import ctypes

import numpy as np
import pytest
import torch

from apophis_gb300 import _capi, hydro, problems

pytestmark = pytest.mark.gpu


def _noalloc(md, cfg, dt_dev):
    nx = (ctypes.c_int * 3)(*cfg.block_nx)
    dx = (ctypes.c_double * 3)(*cfg.dx)
    return _capi.load().aph_hydro_estimate_timestep_noalloc(
        ctypes.c_void_p(md.prim[0].data_ptr()), ctypes.c_void_p(md.cons[0].data_ptr()), nx,
        cfg.ng, cfg.ndim, dx, cfg.gm1, cfg.cfl, ctypes.c_void_p(dt_dev.data_ptr()),
        hydro.stream_handle())


@pytest.mark.parametrize("case", ["kh3d", "kh2d", "sod"])
def test_noalloc_dt_matches_regular_entry_point(cuda, case):
    if case == "kh3d":
        cfg, cons = problems.kh3d(n=48, block=48, ng=4)
    elif case == "kh2d":
        cfg, cons = problems.kh2d(n=256, block=256, ng=3, recon="ppm", rsolver="hllc")
    else:
        cfg, cons = problems.sod(nx=256)
    md = hydro.MeshData(cfg, exact=False)
    md.set_cons(cons)
    hydro.FillGhosts(md)
    hydro.ConsToPrim(md)
    want = hydro.EstimateTimestep(md)
    out = torch.full((2,), -1.0, dtype=torch.float64, device="cuda")
    for k in range(2):  # two calls in a row reuse the shared scratch
        assert _noalloc(md, cfg, out[k:]) == _capi.APH_OK, _capi.load().aph_last_error()
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    assert np.all(np.abs(got - want) <= 1e-13 * want), (got, want)
    assert got[0] == got[1]


def test_noalloc_rejects_blocks_above_the_maximum(cuda):
    cfg, cons = problems.kh3d(n=16, block=16, ng=4)
    md = hydro.MeshData(cfg, exact=False)
    nx = (ctypes.c_int * 3)(128, 128, 128)  # 2M cells > APH_NOALLOC_MAX_CELLS
    dx = (ctypes.c_double * 3)(*cfg.dx)
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    lib = _capi.load()
    st = lib.aph_hydro_estimate_timestep_noalloc(
        ctypes.c_void_p(md.prim[0].data_ptr()), ctypes.c_void_p(md.cons[0].data_ptr()), nx, 4, 3,
        dx, cfg.gm1, cfg.cfl, ctypes.c_void_p(out.data_ptr()), hydro.stream_handle())
    assert st == 1 and b"at most" in lib.aph_last_error()
    # extents whose product would overflow 64 bits are refused too
    nx = (ctypes.c_int * 3)(2 ** 31 - 1, 2 ** 31 - 1, 2 ** 31 - 1)
    st = lib.aph_hydro_estimate_timestep_noalloc(
        ctypes.c_void_p(md.prim[0].data_ptr()), ctypes.c_void_p(md.cons[0].data_ptr()), nx, 4, 3,
        dx, cfg.gm1, cfg.cfl, ctypes.c_void_p(out.data_ptr()), hydro.stream_handle())
    assert st == 1 and b"at most" in lib.aph_last_error()
