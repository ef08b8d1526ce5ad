"""The minimal-surface oracle (oracle/minimal_oracle.c + tests/_ms_oracle.py)
pinned against the reference's regression outputs c/ch7/output/minimal.test*
(tests/golden/minimal_goldens.json), and its Jacobian against differences of
the residual."""
import json
import os

import numpy as np
import pytest

import _ms_oracle as ms

GOLD = {r["test"]: r for r in json.load(open(os.path.join(os.path.dirname(__file__), "golden",
                                                          "minimal_goldens.json")))}


def test_golden_1_catenoid_newton_history_and_error():
    """-snes_fd_color -ms_catenoid_c 2.0 -da_refine 1 (5 x 5): the reference
    solves each Newton step to KSP rtol 1e-5; the oracle solves exactly, so the
    first norm agrees to the printed digits, the following ones to the size of
    the reference's linear-solve error, and the converged error exactly."""
    gold = GOLD[1]
    levels, g, u, err = ms.solve(refine=1, c=2.0)
    r = levels[0]
    assert (g.mx, g.my) == tuple(gold["grid"])
    assert r["its"] == gold["snes_its"][0] and ms.REASONS[r["reason"]] == gold["snes_reasons"][0]
    norms = [float(v) for v in gold["snes_norms"]]
    assert "%g" % r["fnorms"][0] == gold["snes_norms"][0]
    for k in (1, 2, 3, 4):
        assert abs(r["fnorms"][k] - norms[k]) <= 3e-3 * norms[k], k
    assert r["fnorms"][5] < 1e-8 * r["fnorms"][0] and norms[5] < 1e-8 * norms[0]
    assert "%.5e" % err == gold["errinf"]


def test_golden_3_grid_sequence_areas_and_error():
    """-snes_grid_sequence 2 -ms_monitor -ms_quaddegree 2 (3x3 -> 5x5 -> 9x9):
    Newton iterations per grid, every monitored area / diffusivity bound, and
    the final error."""
    gold = GOLD[3]
    levels, g, u, err = ms.solve(grid_sequence=2, monitor_degree=2)
    assert [r["its"] for r in levels] == gold["snes_its"]
    got = [a for r in levels for a in r["areas"]]
    assert len(got) == len(gold["areas"])
    for (a, lo, hi), (ga, glo, ghi) in zip(got, gold["areas"]):
        assert abs(a - ga) <= 1e-7                       # intermediate iterates: reference's inexact steps
        assert "%.4f" % lo == "%.4f" % glo and "%.4f" % hi == "%.4f" % ghi
    # converged iterates agree to every printed digit
    for r, k in zip(levels, (5, 9, 13)):
        assert "%.8f" % r["areas"][-1][0] == "%.8f" % gold["areas"][k][0]
    assert "%.5e" % err == gold["errinf"]


def test_golden_4_tent_grid_sequence_iterations():
    gold = GOLD[4]
    levels, g, u, err = ms.solve(grid_sequence=2, problem=ms.TENT)
    assert [r["its"] for r in levels] == gold["snes_its"]
    assert [ms.REASONS[r["reason"]] for r in levels] == gold["snes_reasons"]
    assert err is None and (g.mx, g.my) == tuple(gold["grid"])


def test_golden_2_q0_is_the_five_point_laplacian():
    """-ms_q 0 (test 2) turns the equation into Laplace's: the Jacobian is the
    5-point stencil with fish's 2D scaling and identity boundary rows (the
    reference's CG iteration counts there depend on PETSc's ILU and are not
    restated)."""
    g = ms.grid(9, ms.TENT, q=0.0)
    J = ms.jacobian(g, ms.initial(g)).toarray()
    n = 4 * 9 + 4
    row = J[n].reshape(9, 9)
    assert row[4, 4] == pytest.approx(4.0)
    assert row[4, 3] == row[4, 5] == row[3, 4] == row[5, 4] == pytest.approx(-1.0)
    assert row[3, 3] == row[5, 5] == row[3, 5] == row[5, 3] == 0.0
    assert J[0, 0] == 1.0 and np.count_nonzero(J[0]) == 1
    assert GOLD[2]["grid"] == [9, 9] and GOLD[2]["problem"] == "tent"


@pytest.mark.parametrize("problem,q,c", [(ms.CATENOID, -0.5, 1.1), (ms.CATENOID, -0.5, 2.0), (ms.TENT, -0.5, 1.0),
                                         (ms.TENT, 0.3, 1.0), (ms.CATENOID, 0.0, 1.5)])
def test_jacobian_is_the_derivative_of_the_residual(problem, q, c):
    rng = np.random.default_rng(7)
    g = ms.grid(17, problem, q=q, c=c)
    u = ms.initial(g) + 0.2 * rng.standard_normal(17 * 17)
    v = rng.standard_normal(17 * 17)
    h = 1e-6
    fd = (ms.residual(g, u + h * v) - ms.residual(g, u - h * v)) / (2 * h)
    jv = ms.jv(g, u, v)
    assert np.max(np.abs(jv - fd)) <= 1e-7 * np.max(np.abs(fd))
    assert np.allclose(ms.jacobian(g, u) @ v, jv, rtol=0, atol=1e-13 * np.max(np.abs(jv)))


def test_interpolation_is_exact_for_bilinear_functions():
    gc, gf = ms.grid(5), ms.grid(9)
    xc = np.linspace(0, 1, 5)
    xf = np.linspace(0, 1, 9)
    f = lambda x, y: 1.0 + 2.0 * x - 3.0 * y + 0.5 * x * y
    uc = f(xc[None, :], xc[:, None]).ravel()
    uf = ms.interpolate(gc, uc, gf)
    assert np.allclose(uf, f(xf[None, :], xf[:, None]).ravel(), atol=1e-14)


def test_exact_catenoid_has_small_residual_and_converges_with_h():
    """FormExactFromG: the continuum catenoid is not the discrete solution;
    the discrete error shrinks like h^2."""
    errs = []
    for m in (9, 17, 33):
        levels, g, u, err = ms.solve(base=m)
        errs.append(err)
    assert errs[0] / errs[1] > 3.0 and errs[1] / errs[2] > 3.0


BRATU = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "bratu_goldens.json")))[0]


def test_bratu_golden_first_norm_and_error():
    """c/ch7/solns/output/bratu2D.test1 (9 x 9, Liouville data): the first
    residual norm to every printed digit; the reference's final iterate (FAS +
    nonlinear Gauss-Seidel, stopped at ||F|| = 8.9e-9) has an error within
    1e-7 of the discrete solution's, which the oracle's Newton reaches."""
    levels, model, u, err = ms.bratu_solve(refine=2, exact=True)
    assert "%g" % levels[0]["fnorms"][0] == BRATU["snes_norms"][0]
    assert (model.mx, model.my) == tuple(BRATU["grid"])
    assert abs(err - float(BRATU["errinf"])) <= 1e-7
    assert levels[0]["reason"] == 3 and levels[0]["its"] == 3


def test_bratu_jacobian_is_the_derivative():
    rng = np.random.default_rng(5)
    for lam, exact in ((1.0, True), (5.0, False)):
        b = ms.Bratu(17, lam, exact)
        u = 0.3 * rng.standard_normal(17 * 17)
        v = rng.standard_normal(17 * 17)
        h = 1e-6
        fd = (b.residual(u + h * v) - b.residual(u - h * v)) / (2 * h)
        assert np.max(np.abs(b.jacobian(u) @ v - fd)) <= 1e-7 * np.max(np.abs(fd))


def test_bratu_error_is_second_order():
    errs = [ms.bratu_solve(refine=r, exact=True, rtol=1e-12)[3] for r in (3, 4, 5)]
    assert errs[0] / errs[1] > 3.5 and errs[1] / errs[2] > 3.5


def test_newton_krylov_baseline_reaches_the_newton_solution():
    """The CPU Newton-Krylov-multigrid solve (the minimal-surface leg's CPU
    baseline) converges on every grid of a sequence and ends at the solution
    of the exact-Newton oracle."""
    u, rep = ms.nk_solve(base=9, grid_sequence=3, rtol=1e-10)
    assert rep.ngrids == 4 and all(rep.reason[k] > 0 for k in range(4))
    lv, g, uo, err = ms.solve(base=9, grid_sequence=3, rtol=1e-10)
    assert np.max(np.abs(u - uo)) <= 1e-7
    assert abs(rep.errinf - err) <= 1e-6 * err
