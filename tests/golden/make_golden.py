"""Generate the golden fixtures under tests/golden/ from the reference's own tests.

Run in the build container only (it reads the reference checkout as text; nothing at
test time reads the reference):

    python tests/golden/make_golden.py /path/to/apophis

sod_exact_t0245.txt -- the exact Sod solution embedded in
    tst/regression/test_suites/riemann_hydro/riemann_hydro.py:192-272
    (columns x, rho, v, p at t = 0.245 for the interface at x = 1 on [0, 2]; the
    +1 shift of line 272 is applied).
pins.json -- the reference's numeric thresholds: the Sod check threshold
    (riemann_hydro.py:147-151) and the linear-wave RMS-L1 bound (convergence.py:130).
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref):
    src = open(os.path.join(ref, "tst/regression/test_suites/riemann_hydro/riemann_hydro.py")).read()
    block = re.search(r'sod_solution = """(.*?)"""', src, re.S).group(1)
    rows = []
    for line in block.strip().splitlines():
        vals = [float(v) for v in line.split()]
        vals[0] += 1.0  # x_ex = x_ex + 1.0 (riemann_hydro.py:272)
        rows.append(vals)
    with open(os.path.join(HERE, "sod_exact_t0245.txt"), "w") as f:
        f.write("# x rho v p  (exact Sod solution, t=0.245, x0=1; from riemann_hydro.py:192-272)\n")
        for r in rows:
            f.write("%.16e %.16e %.16e %.16e\n" % tuple(r))
    conv = open(os.path.join(ref, "tst/regression/test_suites/convergence/convergence.py")).read()
    lw = float(re.search(r"data\[-1, 4\] > ([0-9.e+-]+)", conv).group(1))
    sod_thr = float(re.search(r"\(rho_check - rho\) > ([0-9.]+)", src).group(1))
    with open(os.path.join(HERE, "pins.json"), "w") as f:
        json.dump({"linear_wave_rms_l1_max": lw, "linear_wave_config": "vl2 plm hllc 128x64x64",
                   "sod_exact_threshold": sod_thr, "sod_tlim": 0.245}, f, indent=1)
    print("wrote", len(rows), "rows; pins", lw, sod_thr)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the reference project>")
    main(sys.argv[1])
