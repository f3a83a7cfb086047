"""The CUDA engine of the sharded step (needs a GPU): the batched stepper driven stage by
stage with every ghost cell filled by the halo exchange (aph_stepper_stage with
APH_STAGE_GHOSTS_GIVEN, aph_stepper_local_dt, aph_stepper_end_step).  On one GPU a shard is
the whole mesh, so the exchange moves every ghost value within the rank; three RK2 steps must
equal the stepper's own steps (and the oracle's) bit for bit.  The two-rank orchestration of
the same step is tested on CPU processes (test_shard_gloo.py)."""
import numpy as np
import pytest

from apophis_gb300 import problems, shard
from apophis_gb300.stepper import Stepper
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["kh2d", "rt2d", "kh3d"])
def test_sharded_steps_on_one_gpu_match_the_stepper(cuda, name):
    if name == "kh2d":
        cfg, cons = problems.kh2d(n=64, block=16, ng=3, recon="ppm", rsolver="hllc")
    elif name == "rt2d":
        cfg, cons = problems.rt2d(nx=16, ny=48, block=(8, 16), ng=4)
    else:
        cfg, cons = problems.kh3d(n=32, block=16, ng=4)
    parts = shard.partition(cfg, 1)
    eng = shard.GpuShard(cfg, parts, 0, cons[parts[0]], exact=True)
    ref = Stepper(cfg, cons, exact=True)
    assert eng.status() == ref.status()
    shard.step(eng, 3)
    ref.step(3)
    assert eng.status() == ref.status()
    sk, sj, si = cfg.interior
    got = eng.cons.cpu().numpy()[:, :, sk, sj, si]
    assert np.array_equal(got, ref.state()[parts[0]][:, :, sk, sj, si])
    m = O.Mesh(cfg)
    m.set_cons(cons)
    m.run(nsteps=3)
    assert np.array_equal(got, m.get("cons")[parts[0]][:, :, sk, sj, si])
    eng.close()
    ref.close()


def test_stage_entry_points_reject_bad_arguments(cuda):
    from apophis_gb300 import _capi
    cfg, cons = problems.kh2d(n=32, block=16, ng=3, recon="ppm", rsolver="hllc")
    st = Stepper(cfg, cons, exact=True)
    lib = _capi.load()
    assert lib.aph_stepper_stage(st.h, 2, 0, None) == 1       # RK2 has stages 0 and 1
    assert lib.aph_stepper_stage(st.h, 0, 0x10, None) == 1    # unknown flag
    assert lib.aph_stepper_end_step(st.h, -1.0, None) == 1    # estimates are positive
    st.close()
