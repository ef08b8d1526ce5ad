"""Regenerate tests/golden/minimal_goldens.json and bratu_goldens.json from the
reference's regression files: the run lines of c/ch7/makefile and
c/ch7/solns/makefile (options, MPI process count) and the expected stdout in
c/ch7/output/minimal.test{1..4} and c/ch7/solns/output/bratu2D.test1.  Run where the reference
tree is mounted:

    python tests/golden/make_minimal_goldens.py /path/to/p4pdes
"""
import json
import os
import re
import sys


def main(ref):
    mk = open(os.path.join(ref, "c", "ch7", "makefile")).read()
    runs = re.findall(r'runminimal_(\d+):\s*\n\s*-@\.\./testit\.sh minimal "([^"]*)" (\d+) (\d+)', mk)
    out = []
    for num, opts, nproc, testn in runs:
        text = open(os.path.join(ref, "c", "ch7", "output", "minimal.test%s" % testn)).read()
        rec = {"test": int(testn), "args": opts.split(), "nproc": int(nproc), "stdout": text}
        rec["snes_norms"] = re.findall(r"\d+ SNES Function norm (\S+)", text)
        rec["snes_its"] = [int(v) for v in re.findall(r"Nonlinear solve converged due to \S+ iterations (\d+)", text)]
        rec["snes_reasons"] = re.findall(r"Nonlinear solve converged due to (\S+)", text)
        rec["ksp_its"] = [int(v) for v in re.findall(r"Linear solve converged due to \S+ iterations (\d+)", text)]
        rec["areas"] = [[float(a), float(b), float(c)] for a, b, c in
                        re.findall(r"area = (\S+); (\S+) <= D <= (\S+)", text)]
        m = re.search(r"done on (\d+) x (\d+) grid and problem (\w+)", text)
        rec["grid"], rec["problem"] = [int(m.group(1)), int(m.group(2))], m.group(3)
        m = re.search(r"error \|u-uexact\|_inf = (\S+)", text)
        rec["errinf"] = m.group(1) if m else None
        out.append(rec)
    out.sort(key=lambda r: r["test"])
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "minimal_goldens.json"), "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    print("wrote %d records" % len(out))
    # c/ch7/solns/bratu2D.c's regression run (FAS + nonlinear Gauss-Seidel)
    mk = open(os.path.join(ref, "c", "ch7", "solns", "makefile")).read()
    runs = re.findall(r'runbratu2D_(\d+):\s*\n\s*-@\.\./\.\./testit\.sh bratu2D "([^"]*)" (\d+) (\d+)', mk)
    bout = []
    for num, opts, nproc, testn in runs:
        text = open(os.path.join(ref, "c", "ch7", "solns", "output", "bratu2D.test%s" % testn)).read()
        rec = {"test": int(testn), "args": opts.split(), "nproc": int(nproc), "stdout": text}
        rec["snes_norms"] = re.findall(r"\d+ SNES Function norm (\S+)", text)
        rec["snes_its"] = [int(v) for v in re.findall(r"Nonlinear solve converged due to \S+ iterations (\d+)", text)]
        m = re.search(r"done on (\d+) x (\d+) grid:\s+error \|u-uexact\|_inf = (\S+)", text)
        rec["grid"], rec["errinf"] = [int(m.group(1)), int(m.group(2))], m.group(3)
        bout.append(rec)
    with open(os.path.join(here, "bratu_goldens.json"), "w") as f:
        json.dump(bout, f, indent=1)
        f.write("\n")
    print("wrote %d bratu records" % len(bout))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python %s <path of the p4pdes source tree>" % sys.argv[0])
    main(sys.argv[1])
