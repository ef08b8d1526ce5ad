"""GPU tests of the Liouville-Bratu client (c/ch7/solns/bratu2D.c): the
residual call-back against the oracle, Newton solves against the oracle's
Newton and the reference's regression output, and the C driver."""
import json
import os
import subprocess

import numpy as np
import pytest

import _ms_oracle as ms

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = json.load(open(os.path.join(ROOT, "tests", "golden", "bratu_goldens.json")))[0]


@pytest.mark.parametrize("lam,exact", [(1.0, True), (1.0, False), (6.0, False)])
def test_residual_callback_matches_oracle(cuda, lam, exact):
    import torch
    import p4pdes_gb300 as fg
    m = 33
    u = 0.5 * np.random.default_rng(4).standard_normal(m * m)
    want = ms.Bratu(m, lam, exact).residual(u)
    inf = fg.Info()
    inf.dim, inf.mx, inf.my, inf.mz = 2, m, m, 1
    inf.xm, inf.ym, inf.zm = m, m, 1
    inf.xmax[0] = inf.xmax[1] = 1.0
    ud = torch.from_numpy(u.reshape(m, m)).cuda()
    F = torch.empty_like(ud)
    fg.BratuFunctionLocal(inf, ud, F, lam, exact)
    assert np.max(np.abs(F.cpu().numpy().ravel() - want)) <= 1e-13 * np.max(np.abs(want))


def solve(args):
    import p4pdes_gb300 as fg
    o = fg.bratu_options(args)
    return fg.ms_solve(o)


def test_golden_grid_first_norm_and_error(cuda):
    u, rep = solve("-lb_exact -da_refine 2")
    assert "%g" % rep.fnorm[0][0] == GOLD["snes_norms"][0]
    assert rep.reason[0] == 3 and rep.its[0] == 3
    assert abs(rep.errinf - float(GOLD["errinf"])) <= 1e-7


@pytest.mark.parametrize("args,refine,gs,lam,exact", [
    ("-lb_exact -da_refine 6 -snes_rtol 1e-10", 6, 0, 1.0, True),
    ("-lb_lambda 6.0 -da_refine 5 -snes_rtol 1e-10", 5, 0, 6.0, False),
    ("-lb_exact -da_refine 3 -snes_grid_sequence 3 -snes_rtol 1e-10", 3, 3, 1.0, True),
])
def test_solution_matches_oracle_newton(cuda, args, refine, gs, lam, exact):
    u, rep = solve(args)
    assert all(rep.reason[k] > 0 for k in range(rep.ngrids))
    lv, model, uo, err = ms.bratu_solve(refine=refine, grid_sequence=gs, lam=lam, exact=exact, rtol=1e-10)
    assert u.shape == (model.my, model.mx)
    assert np.max(np.abs(u.ravel() - uo)) <= 1e-8 * max(np.max(np.abs(uo)), 1.0)
    fn = np.linalg.norm(model.residual(u.ravel()))
    last = rep.ngrids - 1
    assert fn <= 1e-10 * rep.fnorm[last][0] * 1.01 or rep.reason[last] == 4
    if exact:  # the errors differ by at most the difference of the solutions
        assert abs(rep.errinf - err) <= 1e-8 * max(np.max(np.abs(uo)), 1.0)


def test_driver_lines(cuda):
    exe = os.path.join(ROOT, "p4pdes_gb300", "bin", "bratu2D")
    p = subprocess.run([exe, "-lb_exact", "-snes_converged_reason", "-snes_monitor_short", "-da_refine", "2"],
                       stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert p.returncode == 0, p.stderr
    lines = p.stdout.splitlines()
    want = GOLD["stdout"].splitlines()
    assert lines[0].rstrip() == want[0].rstrip()                   # 0 SNES Function norm 9.04754
    assert lines[-2] == "Nonlinear solve converged due to CONVERGED_FNORM_RELATIVE iterations 3"
    assert lines[-1].startswith("done on 9 x 9 grid:   error |u-uexact|_inf = 3.16")
    p = subprocess.run([exe, "-snes_type", "fas"], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert p.returncode == 7                                        # FAS is not offered
