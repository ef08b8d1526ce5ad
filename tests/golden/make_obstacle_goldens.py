"""Regenerate tests/golden/obstacle_goldens.json from the reference's regression
files: the run lines of c/ch12/makefile (options, MPI process count) and the
expected stdout in c/ch12/output/obstacle.test{1..4}.  Run where the reference
tree is mounted:

    python tests/golden/make_obstacle_goldens.py /path/to/p4pdes
"""
import json
import os
import re
import sys


def main(ref):
    mk = open(os.path.join(ref, "c", "ch12", "makefile")).read()
    runs = re.findall(r'runobstacle_(\d+):\s*\n(?:#[^\n]*\n)*\s*-@\.\./testit\.sh obstacle "([^"]*)" (\d+) (\d+)', mk)
    out = []
    for num, opts, nproc, testn in runs:
        text = open(os.path.join(ref, "c", "ch12", "output", "obstacle.test%s" % testn)).read()
        rec = {"test": int(testn), "args": opts.split(), "nproc": int(nproc), "stdout": text}
        rec["snes_norms"] = re.findall(r"\d+ SNES Function norm (\S+)", text)
        rec["snes_its"] = [int(v) for v in re.findall(r"Nonlinear solve converged due to \S+ iterations (\d+)", text)]
        m = re.search(r"done on (\d+) x (\d+) grid \.\.\. (\S+), SNES iters = (\d+), last KSP iters = (\d+)", text)
        rec["grid"], rec["reason"], rec["its"], rec["last_ksp_its"] = \
            [int(m.group(1)), int(m.group(2))], m.group(3), int(m.group(4)), int(m.group(5))
        m = re.search(r"errors: av \|u-uexact\| = (\S+), \|u-uexact\|_inf = (\S+), active area error = (\S+)%", text)
        rec["err1"], rec["errinf"], rec["area_err_pct"] = m.group(1), m.group(2), m.group(3)
        out.append(rec)
    out.sort(key=lambda r: r["test"])
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "obstacle_goldens.json"), "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    print("wrote %d records" % len(out))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python %s <path of the p4pdes source tree>" % sys.argv[0])
    main(sys.argv[1])
