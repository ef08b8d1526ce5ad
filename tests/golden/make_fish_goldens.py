"""Regenerate tests/golden/fish_goldens.json from the reference's regression
files: the run lines of c/ch6/makefile (options, MPI process count) and the
expected stdout in c/ch6/output/fish.test{1..8}.  Run where the reference tree
is mounted:

    python tests/golden/make_fish_goldens.py /path/to/p4pdes
"""
import json
import os
import re
import sys


def main(ref):
    mk = open(os.path.join(ref, "c", "ch6", "makefile")).read()
    runs = re.findall(r'runfish_(\d+):\s*\n\s*-@\.\./testit\.sh fish "([^"]*)" (\d+) (\d+)', mk)
    out = []
    for num, opts, nproc, testn in runs:
        path = os.path.join(ref, "c", "ch6", "output", "fish.test%s" % testn)
        text = open(path).read()
        rec = {"test": int(testn), "args": opts.split(), "nproc": int(nproc), "stdout": text}
        m = re.search(r"error \|u-uexact\|_inf = (\S+), \|u-uexact\|_h = (\S+)", text)
        rec["errinf"], rec["err2h"] = m.group(1), m.group(2)
        m = re.search(r"iterations (\d+)", text)
        rec["its"] = int(m.group(1)) if m else None
        m = re.search(r"0 SNES Function norm (\S+)", text)
        rec["snes_norm0"] = m.group(1) if m else None
        m = re.search(r"problem (\S+) on (.*) grid:", text)
        rec["problem"], rec["grid"] = m.group(1), m.group(2)
        out.append(rec)
    out.sort(key=lambda r: r["test"])
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "fish_goldens.json"), "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    print("wrote %d records" % len(out))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python %s <path of the p4pdes source tree>" % sys.argv[0])
    main(sys.argv[1])
