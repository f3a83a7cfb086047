"""Failure paths on the GPU without a fault: a grid barrier that runs out returns
APH_ERR_TIMEOUT and leaves the context usable; a non-finite state is reported as
APH_ERR_STATE; a checkpoint/resume cycle reproduces an uninterrupted run bit for bit."""
import time

import numpy as np
import pytest

from apophis_gb300 import _capi, problems
from apophis_gb300.hydro import stream_handle
from apophis_gb300.stepper import Stepper

pytestmark = pytest.mark.gpu


def test_barrier_timeout_is_reported_and_context_survives(cuda):
    _capi.load()
    t0 = time.perf_counter()
    with pytest.raises(_capi.AphError) as ei:
        _capi.call("aph_diag_barrier_timeout", 0.05, stream_handle())
    assert "TIMEOUT" in str(ei.value) or "gave up" in str(ei.value)
    assert time.perf_counter() - t0 < 5.0
    cfg, cons = problems.kh3d(n=16, block=8, ng=4)
    st = Stepper(cfg, cons, exact=True)
    st.step(2)
    assert st.status()["ncycle"] == 2
    st.close()


def test_nonfinite_state_is_reported(cuda):
    cfg, cons = problems.kh3d(n=16, block=8, ng=4)
    cons = cons.copy()
    sk, sj, si = cfg.interior
    cons[3, 4, 2 + sk.start, 3 + sj.start, 4 + si.start] = np.nan
    st = Stepper(cfg, cons, exact=False, fixed_dt=1e-4)
    st.step(1)
    with pytest.raises(_capi.AphError) as ei:
        st.status()
    assert "NaN" in str(ei.value) or "STATE" in str(ei.value)
    st.close()


def test_checkpoint_resume_is_bit_identical(cuda, tmp_path):
    cfg, cons = problems.kh3d(n=16, block=8, ng=4)
    a = Stepper(cfg, cons, exact=True)
    a.step(10)
    want, sa = a.state(), a.status()
    a.close()
    b = Stepper(cfg, cons, exact=True)
    b.step(5)
    base = str(tmp_path / "ckpt")
    b.save(base)
    b.close()
    c = Stepper.restore(base, cfg)
    c.step(5)
    got, sc = c.state(), c.status()
    c.close()
    sk, sj, si = cfg.interior
    assert np.array_equal(got[:, :, sk, sj, si], want[:, :, sk, sj, si])
    assert sc == sa
