"""The C++ face of the library (include/aph_apophis.hpp): a host program written in the
reference's terms (tests/cpp/sod_tasks.cpp) compiles and links against the library (CPU),
and on the GPU reproduces the oracle's Sod run bit for bit in exact mode."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from apophis_gb300 import _build, problems

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _compile(tmp_path):
    lib = _build.build()
    libdir = os.path.dirname(lib)
    exe = str(tmp_path / "sod_tasks")
    cmd = ["g++", "-std=c++17", "-O2", os.path.join(ROOT, "tests", "cpp", "sod_tasks.cpp"),
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(CUDA, "include"),
           "-L", libdir, "-laph_hydro", "-L", os.path.join(CUDA, "lib64"), "-lcudart",
           "-Wl,-rpath," + libdir, "-Wl,-rpath," + os.path.join(CUDA, "lib64"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_cpp_face_compiles_and_links(tmp_path):
    assert os.path.exists(_compile(tmp_path))


@pytest.mark.gpu
def test_cpp_task_sequence_matches_oracle(cuda, tmp_path):
    from oracle import oracle as O
    exe = _compile(tmp_path)
    cfg, cons = problems.sod(nx=256, recon="plm", rsolver="hlle", integrator="rk2", cfl=0.4)
    assert cfg.ng == 2
    inp, out = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    np.ascontiguousarray(cons[0, :, 0, 0, :]).tofile(inp)
    r = subprocess.run([exe, inp, out, "256", "0.2", "1"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    raw = np.fromfile(out)
    got, (time, ncycle, mass) = raw[:-3].reshape(5, -1), raw[-3:]
    m = O.Mesh(cfg)
    m.set_cons(cons)
    m.run(tlim=0.2)
    st = m.state()
    assert time == st["time"] and int(ncycle) == st["ncycle"]
    g = cfg.ng
    want = m.get("cons")[0, :, 0, 0, :]
    assert np.array_equal(got[:, g:-g], want[:, g:-g])
    assert mass == pytest.approx(O.history(cfg, m.get("cons"))["total_mass"], rel=1e-14)
