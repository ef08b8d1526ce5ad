"""GPU tests of the obstacle client (c/ch12/obstacle.c): the reduced-space
active-set Newton on the GPU against the reference's regression outputs and
the oracle, and the C driver's lines and binary dump."""
import json
import os
import re
import subprocess

import numpy as np
import pytest

import _obs_oracle as ob

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = {r["test"]: r for r in json.load(open(os.path.join(ROOT, "tests", "golden", "obstacle_goldens.json")))}
EXE = os.path.join(ROOT, "p4pdes_gb300", "bin", "obstacle")


def gpu_solve(args):
    import p4pdes_gb300 as fg
    return fg.ms_solve(fg.obstacle_options(args))


def errors(rep):
    return "%.3e" % rep.err1, "%.3e" % rep.errinf, "%.3f" % (100 * rep.active_area_err)


def test_golden_1(cuda):
    """-ksp_rtol 1e-12: the reference's Newton step is exact and it stops after
    2 steps; the FP32 inner solve resolves a step to ~1e-7 relative, so the
    GPU takes one more FP64-residual step (the mixed-precision signature)."""
    gold = GOLD[1]
    u, rep = gpu_solve(gold["args"])
    detail = ([rep.fnorm[0][i] for i in range(rep.its[0] + 1)], [rep.ksp_its[0][i] for i in range(rep.its[0])],
              [rep.ksp_reason[0][i] for i in range(rep.its[0])])
    assert rep.its[0] in (gold["its"], gold["its"] + 1) and rep.reason[0] == 3, detail
    assert ["%g" % rep.fnorm[0][i] for i in range(2)] == gold["snes_norms"][:2]
    assert rep.fnorm[0][rep.its[0]] < 1e-11
    assert errors(rep) == (gold["err1"], gold["errinf"], gold["area_err_pct"])


@pytest.mark.parametrize("test", [3, 4])
def test_goldens_errors(cuda, test):
    gold = GOLD[test]
    u, rep = gpu_solve(gold["args"])
    assert all(rep.reason[k] > 0 for k in range(rep.ngrids))
    assert [rep.m[rep.ngrids - 1]] * 2 == gold["grid"]
    assert errors(rep) == (gold["err1"], gold["errinf"], gold["area_err_pct"])


@pytest.mark.parametrize("args,refine,gs", [("-da_refine 5 -snes_rtol 1e-10", 5, 0),
                                            ("-snes_grid_sequence 6 -snes_rtol 1e-10", 0, 6)])
def test_solution_matches_oracle(cuda, args, refine, gs):
    u, rep = gpu_solve(args)
    levels = ob.run(refine=refine, grid_sequence=gs, rtol=1e-10)
    r = levels[-1]
    assert u.shape == (r["m"], r["m"])
    assert np.max(np.abs(u.ravel() - r["u"])) <= 1e-9
    e1, ei, ae, nact = ob.report(r["m"], r["u"], r["F"])
    assert rep.n_active == nact
    assert abs(rep.err1 - e1) <= 1e-9 and abs(rep.errinf - ei) <= 1e-9


def test_driver_lines_and_dump(cuda, tmp_path):
    gold = GOLD[3]
    p = subprocess.run([EXE] + gold["args"], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert p.returncode == 0, p.stderr
    got, want = p.stdout.splitlines(), gold["stdout"].splitlines()
    assert len(got) == len(want) and got[-1] == want[-1]
    num = re.compile(r"\d+")
    for a, b in zip(got, want):
        assert num.sub("#", a) == num.sub("#", b)  # same lines and indentation; iteration counts aside
    f = tmp_path / "dump.dat"
    p = subprocess.run([EXE, "-da_refine", "2", "-obs_dump_binary", str(f)], stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, text=True)
    assert p.returncode == 0, p.stderr
    assert ("writing u,psi in binary format to %s ..." % f) in p.stdout
    import p4pdes_gb300 as fg
    u, lo = fg.petsc_vec_read(f, 0), fg.petsc_vec_read(f, 1)
    h, X, Y = ob.coords(9)
    assert np.allclose(lo, ob.psi(X, Y).ravel(), rtol=0, atol=1e-15)
    assert np.all(u >= lo - 1e-15)
