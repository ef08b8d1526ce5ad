"""GPU tests of the minimal-surface path (c/ch7/minimal.c): the residual
call-back against the oracle, and the Newton solver (FP32 inner BiCGStab +
Poisson multigrid, FP64 residual and update) against the reference's
regression outputs and the oracle's Newton solution."""
import json
import os
import re
import subprocess

import numpy as np
import pytest

import _ms_oracle as ms

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = {r["test"]: r for r in json.load(open(os.path.join(ROOT, "tests", "golden", "minimal_goldens.json")))}


def info_2d(m, xs=0, ys=0, xm=None, ym=None):
    import p4pdes_gb300 as fg
    inf = fg.Info()
    inf.dim, inf.mx, inf.my, inf.mz = 2, m, m, 1
    inf.xs, inf.ys, inf.zs = xs, ys, 0
    inf.xm, inf.ym, inf.zm = (m - xs if xm is None else xm), (m - ys if ym is None else ym), 1
    inf.xmax[0] = inf.xmax[1] = 1.0
    return inf


@pytest.mark.parametrize("problem,q,c", [(ms.CATENOID, -0.5, 1.1), (ms.TENT, -0.5, 1.0), (ms.CATENOID, 0.3, 2.0),
                                         (ms.TENT, 0.0, 1.0)])
def test_residual_callback_matches_oracle(cuda, problem, q, c):
    import torch
    import p4pdes_gb300 as fg
    m = 33
    g = ms.grid(m, problem, q=q, c=c, H=0.7)
    u = ms.initial(g) + 0.3 * np.random.default_rng(3).standard_normal(m * m)
    want = ms.residual(g, u)
    ctx = fg.MsCtx(problem, q, c, 0.7)
    ud = torch.from_numpy(u.reshape(m, m)).cuda()
    F = torch.full_like(ud, 7.0)
    fg.MinimalFunctionLocal(info_2d(m), ud, F, ctx)
    got = F.cpu().numpy().ravel()
    assert np.max(np.abs(got - want)) <= 1e-13 * np.max(np.abs(want))
    # an owned sub-box writes only its nodes
    F2 = torch.full_like(ud, 7.0)
    fg.MinimalFunctionLocal(info_2d(m, 5, 9, 20, 11), ud, F2, ctx)
    F2 = F2.cpu().numpy()
    box = np.zeros((m, m), bool)
    box[9:20, 5:25] = True
    assert np.all(F2[~box] == 7.0)
    assert np.max(np.abs(F2[box] - want.reshape(m, m)[box])) <= 1e-13 * np.max(np.abs(want))


def run(args):
    import p4pdes_gb300 as fg
    o = fg.ms_options(args)
    u, rep = fg.ms_solve(o)
    return o, u, rep


def test_golden_1_newton_history_and_error(cuda):
    gold = GOLD[1]
    o, u, rep = run(gold["args"])
    assert rep.ngrids == 1 and rep.m[0] == gold["grid"][0]
    assert rep.its[0] == gold["snes_its"][0]
    import p4pdes_gb300 as fg
    assert fg.snes_reason_name(rep.reason[0]) == gold["snes_reasons"][0]
    norms = [float(v) for v in gold["snes_norms"]]
    got = rep.fnorms(0)
    assert "%g" % got[0] == gold["snes_norms"][0]
    for k in (1, 2, 3):
        assert abs(got[k] - norms[k]) <= 3e-3 * norms[k], (k, got[k], norms[k])
    assert got[-1] <= 1e-8 * got[0]
    assert "%.5e" % rep.errinf == gold["errinf"]


def test_golden_3_grid_sequence(cuda):
    gold = GOLD[3]
    o, u, rep = run(gold["args"])
    assert [rep.its[k] for k in range(rep.ngrids)] == gold["snes_its"]
    got = [a for k in range(rep.ngrids) for a in rep.areas(k)]
    assert len(got) == len(gold["areas"])
    for (a, lo, hi), (ga, glo, ghi) in zip(got, gold["areas"]):
        assert abs(a - ga) <= 2e-7
        assert "%.4f" % lo == "%.4f" % glo and "%.4f" % hi == "%.4f" % ghi
    for k, gk in zip(range(3), (5, 9, 13)):
        assert "%.8f" % rep.areas(k)[-1][0] == "%.8f" % gold["areas"][gk][0]
    assert "%.5e" % rep.errinf == gold["errinf"]


def test_golden_4_tent_grid_sequence(cuda):
    gold = GOLD[4]
    o, u, rep = run(gold["args"])
    assert [rep.its[k] for k in range(rep.ngrids)] == gold["snes_its"]
    assert rep.errinf < 0


def test_golden_2_laplace_tent(cuda):
    """q = 0: Laplace's equation with tent data (test 2's grid); the solution
    equals the oracle's to the Newton tolerance."""
    gold = GOLD[2]
    o, u, rep = run(gold["args"])
    assert rep.reason[0] > 0 and [rep.m[0]] * 2 == gold["grid"]
    lv, g, uo, err = ms.solve(refine=2, problem=ms.TENT, q=0.0)
    assert np.max(np.abs(u.ravel() - uo)) <= 1e-7


# Newton from u = 0 inside stalls beyond 33 x 33 (the oracle's exact Newton
# too: its steps shrink to nothing at 65 x 65), so larger grids are reached
# by grid sequencing, as minimal.c recommends.
@pytest.mark.parametrize("args,base,refine,gs", [
    ("-da_refine 4 -snes_rtol 1e-10", 3, 4, 0),
    ("-da_grid_x 33 -da_grid_y 33 -snes_grid_sequence 2 -snes_rtol 1e-10", 33, 0, 2),
    ("-da_refine 2 -snes_grid_sequence 4 -snes_rtol 1e-10", 3, 2, 4),
    ("-da_refine 4 -ms_problem tent -ms_tent_H 0.5 -snes_rtol 1e-10", 3, 4, 0),
])
def test_solution_matches_oracle_newton(cuda, args, base, refine, gs):
    import p4pdes_gb300 as fg
    o, u, rep = run(args)
    for k in range(rep.ngrids):
        assert rep.reason[k] > 0
    kw = {"problem": ms.TENT, "H": 0.5} if "tent" in args else {}
    lv, g, uo, err = ms.solve(base=base, refine=refine, grid_sequence=gs, rtol=1e-10, **kw)
    assert u.shape == (g.my, g.mx)
    scale = np.max(np.abs(uo))
    assert np.max(np.abs(u.ravel() - uo)) <= 1e-8 * scale
    # the residual of the GPU solution, recomputed by the oracle in FP64,
    # is the one the solver reported and meets rtol
    last = rep.ngrids - 1
    fn = np.linalg.norm(ms.residual(g, u.ravel()))
    assert abs(fn - rep.fnorm[last][rep.its[last]]) <= 1e-3 * fn + 1e-14
    assert fn <= 1e-10 * rep.fnorm[last][0]
    if err is not None:
        assert abs(rep.errinf - err) <= 1e-6 * err


def test_reuse_is_deterministic(cuda):
    import p4pdes_gb300 as fg
    o = fg.ms_options("-da_refine 5 -snes_grid_sequence 1")
    with fg.MsSolver(o) as s:
        u1 = np.empty((129, 129))
        u2 = np.empty((129, 129))
        r1 = s.solve(u1)
        r2 = s.solve(u2)
    assert np.array_equal(u1, u2)
    assert r1.fnorms(1) == r2.fnorms(1) and r1.total_ksp_its == r2.total_ksp_its


def driver(args):
    exe = os.path.join(ROOT, "p4pdes_gb300", "bin", "minimal")
    return subprocess.run([exe] + args, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)


@pytest.mark.parametrize("test", [1, 3, 4])
def test_driver_prints_the_reference_lines(cuda, test):
    """The C driver's stdout has the reference's lines: identical where they do
    not depend on the inexact Newton steps (first norm, reasons, converged
    areas, the final line), same count and layout everywhere."""
    gold = GOLD[test]
    p = driver(gold["args"])
    assert p.returncode == 0, p.stderr
    want = gold["stdout"].splitlines()
    got = p.stdout.splitlines()
    assert len(got) == len(want)
    assert got[-1] == want[-1]
    num = re.compile(r"\d+(\.\d*)?(e[-+]\d+)?")
    for a, b in zip(got, want):
        if "Nonlinear solve" in b or " 0 SNES Function norm" in b:
            assert a == b
        else:
            assert num.sub("#", a) == num.sub("#", b)  # same line and indentation, numbers aside


def test_drivers_write_the_solution_as_petsc_binary(cuda, tmp_path):
    """-snes_view_solution binary:FILE writes the final iterate as a PETSc
    binary Vec in natural ordering."""
    import p4pdes_gb300 as fg
    f = tmp_path / "u.dat"
    p = driver(["-da_refine", "3", "-snes_view_solution", "binary:%s" % f])
    assert p.returncode == 0, p.stderr
    u = fg.petsc_vec_read(f)
    lv, g, uo, err = ms.solve(refine=3)
    assert u.size == g.mx * g.my and np.max(np.abs(u - uo)) <= 1e-7
    exe = os.path.join(ROOT, "p4pdes_gb300", "bin", "fish")
    f2 = tmp_path / "fish.dat"
    args = "-fsh_dim 2 -da_refine 4 -pc_type mg -ksp_rtol 1e-12".split()
    p = subprocess.run([exe] + args + ["-snes_view_solution", "binary:%s" % f2], stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, text=True)
    assert p.returncode == 0, p.stderr
    import _oracle as orc
    uref, ref = orc.fish_solve(orc.options(args))
    assert np.max(np.abs(fg.petsc_vec_read(f2) - uref.ravel())) <= 1e-9 * np.max(np.abs(uref))


@pytest.mark.parametrize("args", ["-da_grid_x 33 -da_grid_y 33 -snes_grid_sequence 2 -snes_rtol 1e-10",
                                  "-da_refine 4 -ms_problem tent -ms_tent_H 0.5 -snes_rtol 1e-10",
                                  "-da_refine 3 -pc_type none -snes_rtol 1e-10"])
def test_one_block_inner_solve_matches_the_launch_per_phase_form(cuda, args):
    """On grids of up to 4096 nodes whose preconditioner is one exact coarse
    solve the inner BiCGStab runs as one block (k_bi_block): the same
    iteration and finalisers, dot products summed in another order, so the
    Newton solve takes the same steps and ends at the same solution to the
    Newton tolerance."""
    import p4pdes_gb300 as fg
    o1, u1, r1 = run(args + " -ms_inner_block 1")
    o0, u0, r0 = run(args + " -ms_inner_block 0")
    assert r1.ngrids == r0.ngrids
    for k in range(r0.ngrids):
        assert r1.reason[k] > 0 and r0.reason[k] > 0
        assert r1.its[k] == r0.its[k]
    assert np.max(np.abs(u1 - u0)) <= 1e-8 * np.max(np.abs(u0))


@pytest.mark.parametrize("kind,args", [
    ("minimal", "-da_grid_x 33 -da_grid_y 33 -snes_grid_sequence 3 -snes_rtol 1e-10"),
    ("minimal", "-da_refine 2 -snes_grid_sequence 4 -ms_problem tent -ms_tent_H 0.5 -snes_rtol 1e-10"),
    ("bratu", "-da_refine 7 -snes_rtol 1e-10"),
    ("obstacle", "-da_refine 2 -snes_grid_sequence 5"),
])
def test_persistent_inner_solve_matches_the_launch_per_phase_form(cuda, kind, args):
    """On multigrid grids the inner BiCGStab solve runs as one cooperative
    launch (k_bi_persist, the default up to FISHGPU_MS_PERSIST_POINTS nodes):
    the same iteration, V-cycle values and finalisers as the launch-per-phase
    graphs, the dot products summed in another order, so every grid takes the
    same Newton steps and ends at the same solution to the Newton tolerance."""
    import p4pdes_gb300 as fg
    opts = {"minimal": fg.ms_options, "bratu": fg.bratu_options, "obstacle": fg.obstacle_options}[kind]
    r1 = fg.ms_solve(opts(args))
    r0 = fg.ms_solve(opts(args + " -ms_inner_persist 0"))
    (u1, rep1), (u0, rep0) = r1, r0
    assert rep1.ngrids == rep0.ngrids
    for k in range(rep0.ngrids):
        assert rep1.reason[k] > 0 and rep0.reason[k] > 0
        assert rep1.its[k] == rep0.its[k]
        small = rep0.m[k] ** 2 <= 4096 and rep0.inner_form[k] == 1  # one block (k_bi_block) either way
        assert rep0.inner_form[k] == (1 if small else 0)
        assert rep1.inner_form[k] == (1 if small else 2)
    assert any(rep1.inner_form[k] == 2 for k in range(rep1.ngrids))
    inner1, inner0 = rep1.total_ksp_its, rep0.total_ksp_its
    assert abs(inner1 - inner0) <= max(2, inner0 // 20)
    assert np.max(np.abs(u1 - u0)) <= 1e-8 * np.max(np.abs(u0))
