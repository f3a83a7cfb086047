"""Measure the FP64 instruction throughput of the current GPU (the roofline that binds the
hydro path on GB300).  ``python -m apophis_gb300.fp64_peak`` builds csrc/fp64_peak.cu with
nvcc for sm_103a into _lib/ and prints its table and a JSON summary."""
import json
import os
import re
import subprocess
import sys

from . import _build

SRC = os.path.join(_build.CSRC, "fp64_peak.cu")
BIN = os.path.join(_build.LIBDIR, "fp64_peak")


def build():
    os.makedirs(_build.LIBDIR, exist_ok=True)
    if not os.path.exists(BIN) or os.path.getmtime(BIN) < os.path.getmtime(SRC):
        subprocess.check_call([_build.nvcc()] + _build.ARCH + ["-O3", "-o", BIN, SRC])
    return BIN


def measure():
    out = subprocess.run([build()], capture_output=True, text=True, check=True).stdout
    res = {"raw": out}
    for line in out.splitlines():
        m = re.match(r"(\S+(?:\+\S+)?)\s+([\d.]+) ms\s+([\d.]+) Gop/s\s+([\d.]+) op/clk/SM", line.strip())
        if m:
            res[m.group(1)] = {"gops": float(m.group(3)), "per_clk_per_sm": float(m.group(4))}
    return res


if __name__ == "__main__":
    r = measure()
    sys.stdout.write(r.pop("raw"))
    print(json.dumps(r))
