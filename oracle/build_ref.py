"""Build recipe for ``oracle/_ref/libref_pin.so``: the reference's own reconstruction and
Riemann-solver code compiled from its sources (test infrastructure, not product code).

The reference project as a whole cannot be built here (it needs Kokkos, Parthenon and
singularity-eos through CMake; their submodules are empty).  Its reconstruction headers
(src/recon/{dc,plm,ppm}_simple.hpp) and Riemann solvers (src/hydro/rsolvers/hydro_{none,
hlle,hllc,lhllc}.hpp) are self-contained inline functions, though: compiled where they lie,
against the stand-ins in ``oracle/ref_shim/`` for the handful of Parthenon / Kokkos /
singularity-eos names they use, they give the reference's FP64 arithmetic to pin the oracle
against (``oracle/ref_pin.cpp`` is the C interface; ``tests/test_ref_pin.py`` the check).
No reference source is copied: the compiler reads it from the reference checkout, whose
path is the first argument, or ``$APH_REFERENCE``, or ``/root/reference``.  The output stays
out of version control.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "ref_pin.cpp")
SHIM = os.path.join(HERE, "ref_shim")
OUT_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT_DIR, "libref_pin.so")

# the oracle's own flags: no fused multiply-add, no fast math
FLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-w"]

REF_HEADERS = ["src/main.hpp", "src/recon/dc_simple.hpp", "src/recon/plm_simple.hpp",
               "src/recon/ppm_simple.hpp", "src/hydro/rsolvers/rsolvers.hpp",
               "src/hydro/rsolvers/hydro_none.hpp", "src/hydro/rsolvers/hydro_hlle.hpp",
               "src/hydro/rsolvers/hydro_hllc.hpp", "src/hydro/rsolvers/hydro_lhllc.hpp"]


def reference_path(arg=None):
    return arg or os.environ.get("APH_REFERENCE") or "/root/reference"


def available(ref=None):
    ref = reference_path(ref)
    return all(os.path.exists(os.path.join(ref, h)) for h in REF_HEADERS)


def build(ref=None, force=False):
    """Compile the pin library; returns its path, or None when the reference is absent."""
    ref = reference_path(ref)
    if not available(ref):
        return LIB if os.path.exists(LIB) else None
    deps = [SRC] + [os.path.join(ref, h) for h in REF_HEADERS]
    for root, _, files in os.walk(SHIM):
        deps += [os.path.join(root, f) for f in files]
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps)):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++"] + FLAGS + ["-I", SHIM, "-I", os.path.join(ref, "src"), SRC,
                                             "-o", tmp])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else None, force=True))
