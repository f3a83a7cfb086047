"""Refined-mesh oracle and face tables (CPU only).

The refined-mesh oracle is pinned to the uniform oracle (itself pinned to the reference's
Sod table and linear-wave convergence) by running an unrefined mesh through both; the
cross-level ghost map is checked on fields it reproduces exactly; the flux correction by
conservation to round-off.
"""
import numpy as np
import pytest

from apophis_gb300 import amr, problems
from apophis_gb300.amr import FACE_BOUNDARY, FACE_COARSER, FACE_FINER, FACE_SAME
from oracle import oracle as O


def _interior(cfg, flat, b):
    ng = cfg.ng
    return cfg.block_view(flat, b)[:, 0, ng:-ng, ng:-ng]


def _totals(cfg, flat):
    tot = np.zeros(5)
    for b, B in enumerate(cfg.blocks):
        tot += _interior(cfg, flat, b).sum(axis=(1, 2)) * B.dx[0] * B.dx[1]
    return tot


def test_rt_amr_face_tables():
    cfg, cons = amr.rt2d_amr()
    assert cfg.nblocks == 1440
    assert cfg.level_counts() == {0: 160, 1: 256, 2: 1024}
    assert cfg.zones() == 491520
    opp = [1, 0, 3, 2]
    kinds = {k: 0 for k in range(4)}
    for b, B in enumerate(cfg.blocks):
        for f in range(4):
            k = B.face_kind[f]
            kinds[k] += 1
            for n in B.face_nbr[f]:
                N = cfg.blocks[n]
                if k == FACE_SAME:
                    assert N.level == B.level and N.face_nbr[opp[f]] == [b]
                elif k == FACE_FINER:
                    assert N.level == B.level + 1 and N.face_kind[opp[f]] == FACE_COARSER
                    assert N.face_nbr[opp[f]] == [b]
                elif k == FACE_COARSER:
                    assert N.level == B.level - 1 and N.face_kind[opp[f]] == FACE_FINER
                    assert b in N.face_nbr[opp[f]]
            if k == FACE_BOUNDARY:
                assert f >= 2  # x is periodic, y has walls
    assert kinds == {FACE_SAME: 5472, FACE_COARSER: 192, FACE_FINER: 80, FACE_BOUNDARY: 16}


@pytest.mark.parametrize("recon,rsolver,integrator", [("ppm", "hllc", "rk2"),
                                                      ("plm", "hlle", "rk3"),
                                                      ("plm", "hllc", "vl2")])
def test_unrefined_amr_oracle_matches_uniform_oracle(recon, rsolver, integrator):
    ng = 4 if recon == "ppm" else 2
    cfg, cons = problems.kh2d(n=64, block=16, ng=ng, recon=recon, rsolver=rsolver,
                              integrator=integrator)
    ref = O.Mesh(cfg)
    ref.set_cons(cons)
    ref.run(nsteps=5)
    acfg = amr.uniform_as_amr(cfg)
    m = O.AmrMesh(acfg)
    m.set_cons(np.ascontiguousarray(cons).reshape(-1))
    m.run(nsteps=5)
    assert m.state() == ref.state()
    got = m.get().reshape(cfg.pack_shape(5))
    want = ref.get()
    s = (slice(None), slice(None), slice(None), slice(ng, -ng), slice(ng, -ng))
    assert np.array_equal(got[s], want[s])


@pytest.mark.parametrize("d", [0, 1])
def test_ghost_map_reproduces_linear_fields(d):
    """A field linear in x_d is reproduced exactly in the ghosts of every x_d face that does
    not wrap around the periodic domain: copies, 2x2 restriction and minmod prolongation are
    all exact on it."""
    cfg, _ = amr.small_test_mesh()
    cons = np.zeros(cfg.flat_size(5))
    f = lambda x, y: 3.0 + 0.7 * (x if d == 0 else y)  # noqa: E731
    coef = [1.0, 0.01, -0.02, 0.0, 10.0]  # positive pressure: ConsToPrim leaves cons alone
    ng = cfg.ng
    for b, B in enumerate(cfg.blocks):
        x, y = cfg.cell_centers(b)
        v = cfg.block_view(cons, b)
        for q in range(5):
            v[q, 0, ng:-ng, ng:-ng] = f(x, y) * coef[q]
    m = O.AmrMesh(cfg)
    m.set_cons(cons)
    got = m.get()
    checked = 0
    for b, B in enumerate(cfg.blocks):
        v = cfg.block_view(got, b)
        N = cfg.base_nx[d] << B.level
        for s in range(2):
            if (s == 0 and B.origin[d] == 0) or (s == 1 and B.origin[d] + B.nx[d] == N):
                continue
            for k in range(ng):
                a = -1 - k if s == 0 else B.nx[d] + k
                g = B.origin[d] + a
                xc = cfg.xmin[d] + (g + 0.5) * B.dx[d]
                want = 3.0 + 0.7 * xc
                for t in range(B.nx[1 - d]):
                    idx = [0, 0]
                    idx[d], idx[1 - d] = ng + a, ng + t
                    for q in range(5):
                        assert abs(v[q, 0, idx[1], idx[0]] - want * coef[q]) < 1e-13, (b, s, k, t, q)
                    checked += 1
    assert checked > 1000


def test_refined_oracle_conserves():
    cfg, cons = amr.small_test_mesh()
    m = O.AmrMesh(cfg)
    m.set_cons(cons)
    t0 = _totals(cfg, m.get())
    m.run(nsteps=10)
    t1 = _totals(cfg, m.get())
    scale = np.array([t0[0], abs(t0[1]) + t0[0], abs(t0[2]) + t0[0], 1.0, t0[4]])
    assert np.all(np.abs(t1 - t0) <= 1e-13 * scale), (t1 - t0) / scale


def test_conservation_check_has_teeth():
    """Without the coarse-fine correction the same run leaks mass well above round-off."""
    cfg, cons = amr.small_test_mesh()
    m = O.AmrMesh(cfg)
    m.plant_no_correction()
    m.set_cons(cons)
    t0 = _totals(cfg, m.get())
    m.run(nsteps=10)
    t1 = _totals(cfg, m.get())
    assert abs(t1[0] - t0[0]) > 1e-9 * t0[0]


def _corrupt(cfg, edit):
    table = amr.amr_table(cfg)
    edit(table)
    return table


def test_face_table_check_accepts_meshes():
    for cfg, _ in (amr.rt2d_amr(), amr.small_test_mesh()):
        amr.check_table(cfg)


def test_face_table_check_rejects_bad_tables():
    from apophis_gb300 import _capi
    cfg, _ = amr.small_test_mesh()
    fine = next(b for b, B in enumerate(cfg.blocks) if B.level == 1 and FACE_COARSER in B.face_kind)
    coarse = next(b for b, B in enumerate(cfg.blocks) if FACE_FINER in B.face_kind)
    ff = cfg.blocks[coarse].face_kind.index(FACE_FINER)
    cf = cfg.blocks[fine].face_kind.index(FACE_COARSER)
    same = next(b for b, B in enumerate(cfg.blocks) if B.face_kind[0] == FACE_SAME)

    def set_(b, attr, f, val, n=None):
        def edit(t):
            arr = getattr(t[b], attr)
            if n is None:
                arr[f] = val
            else:
                arr[f][n] = val
        return edit

    bad = [
        set_(same, "face_nbr", 0, cfg.nblocks, 0),           # neighbour out of range
        set_(same, "face_kind", 0, 7),                        # unknown kind
        set_(same, "face_nbr", 0, fine, 0),                   # same-level neighbour on another level
        set_(coarse, "face_count", ff, 1),                    # finer neighbours miss part of the face
        set_(fine, "face_nbr", cf, same, 0),                  # coarser neighbour does not cover it
        set_(same, "face_count", 0, 2),                       # two same-level neighbours
    ]
    for edit in bad:
        with pytest.raises(_capi.AphError):
            amr.check_table(cfg, _corrupt(cfg, edit))
    # odd origin of a fine block at a coarse-fine face
    t = amr.amr_table(cfg)
    t[fine].origin[0] += 1
    t[fine].origin[1] += 1
    with pytest.raises(_capi.AphError):
        amr.check_table(cfg, t)


def test_rt_amr_block_list_is_pinned():
    """The RT pack's block list is deterministic: it equals the committed JSON."""
    import json
    import os
    import sys
    gold = os.path.join(os.path.dirname(__file__), "golden")
    sys.path.insert(0, gold)
    import make_rt_amr_blocks
    want = json.load(open(os.path.join(gold, "rt2d_amr_blocks.json")))
    assert make_rt_amr_blocks.block_list() == want


def test_unrefined_amr_oracle_with_tracers_matches_uniform_oracle():
    """Passive scalars through the refined-mesh oracle: on an unrefined mesh the same bits as
    the uniform oracle (the scalars' ghost map and upwinded fluxes included)."""
    cfg, cons = problems.kh2d_tracers(n=64, block=16, ng=4, recon="ppm", rsolver="hllc")
    ref = O.Mesh(cfg)
    ref.set_cons(cons)
    ref.run(nsteps=5)
    acfg = amr.uniform_as_amr(cfg)
    assert acfg.nvar == 7
    m = O.AmrMesh(acfg)
    m.set_cons(np.ascontiguousarray(cons).reshape(-1))
    m.run(nsteps=5)
    assert m.state() == ref.state()
    got = m.get().reshape(cfg.pack_shape(cfg.nvar))
    s = (slice(None), slice(None), slice(None), slice(4, -4), slice(4, -4))
    assert np.array_equal(got[s], ref.get()[s])


def test_refined_oracle_conserves_tracers():
    cfg, cons = amr.with_tracers(*amr.small_test_mesh(), nscalars=2)
    m = O.AmrMesh(cfg)
    m.set_cons(cons)

    def tracer_mass(flat):
        out = np.zeros(2)
        for b, B in enumerate(cfg.blocks):
            v = cfg.block_view(flat, b)[:, 0, cfg.ng:-cfg.ng, cfg.ng:-cfg.ng]
            out += v[5:7].sum(axis=(1, 2)) * B.dx[0] * B.dx[1]
        return out

    t0 = tracer_mass(m.get())
    m.run(nsteps=10)
    t1 = tracer_mass(m.get())
    assert np.all(np.abs(t1 - t0) <= 1e-13 * np.abs(t0)), (t1 - t0) / t0
