"""Build recipe for the CPU oracle (test infrastructure, not product code).

Compiles ``hydro_oracle.cpp`` into ``oracle/_build/libhydro_oracle.so`` with
``-O2 -ffp-contract=off`` so that no multiply-add is fused: the oracle then
performs the reference's FP64 arithmetic operation by operation, on x86-64 and
on aarch64 alike.  OpenMP parallelises the loops over rows and planes.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "hydro_oracle.cpp")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libhydro_oracle.so")

FLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
         "-fPIC", "-shared"]


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++"] + FLAGS + [SRC, "-o", tmp])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
