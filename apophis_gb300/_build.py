"""Build the CUDA library ``apophis_gb300/_lib/libaph_hydro.so`` for sm_103a.

Each translation unit is compiled with nvcc in parallel and the objects are linked
into one shared library with the shared CUDA runtime (the same runtime PyTorch
loads, so device pointers and streams pass between them).  The exact-arithmetic
unit is built with ``--fmad=false``.
"""
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
OBJDIR = os.path.join(HERE, "_build")
LIB = os.path.join(LIBDIR, "libaph_hydro.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
          "--expt-relaxed-constexpr", "-I" + INCLUDE]

# translation unit -> extra flags
UNITS = {
    "aph_capi.cu": [],
    "aph_ghosts.cu": [],
    "aph_fast.cu": [],
    "aph_exact.cu": ["--fmad=false"],
    "aph_stage_fast.cu": [],
    "aph_stage_exact.cu": ["--fmad=false"],
    "aph_stepper.cu": [],
    "aph_adjoint.cu": [],
    "aph_noalloc.cu": [],
    "aph_history.cu": [],
    "aph_diag.cu": ["--fmad=false"],
}


def nvcc():
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cand = os.path.join(cuda, "bin", "nvcc")
    return cand if os.path.exists(cand) else (shutil.which("nvcc") or "nvcc")


def _sources_digest():
    h = hashlib.sha256()
    for d in (CSRC, INCLUDE):
        for name in sorted(os.listdir(d)):
            if name.endswith((".cu", ".cuh", ".h")):
                with open(os.path.join(d, name), "rb") as f:
                    h.update(name.encode())
                    h.update(f.read())
    h.update(" ".join(ARCH + COMMON).encode())
    h.update(repr(sorted(UNITS.items())).encode())
    return h.hexdigest()


def _compile(unit, extra, verbose):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(OBJDIR, unit.replace(".cu", ".o"))
    cmd = [nvcc()] + ARCH + COMMON + extra + ["-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (unit, " ".join(cmd), r.stderr))
    return obj, r.stderr


def build(force=False, verbose=False, jobs=None):
    """Compile (if sources changed) and return the path of the shared library."""
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)
    stamp = os.path.join(LIBDIR, "libaph_hydro.sha256")
    digest = _sources_digest()
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == digest:
                return LIB
    units = [(u, e) for u, e in UNITS.items() if os.path.exists(os.path.join(CSRC, u))]
    with cf.ThreadPoolExecutor(max_workers=jobs or len(units)) as ex:
        results = list(ex.map(lambda ue: _compile(ue[0], ue[1], verbose), units))
    if verbose:
        for obj, log in results:
            print(obj)
            print(log)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(digest)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force=True, verbose="-v" in sys.argv))
