"""The obstacle-problem oracle (tests/_obs_oracle.py) pinned against the
reference's regression outputs c/ch12/output/obstacle.test* (through
tests/golden/obstacle_goldens.json)."""
import json
import os

import numpy as np
import pytest

import _obs_oracle as ob
import _oracle as orc

GOLD = {r["test"]: r for r in json.load(open(os.path.join(os.path.dirname(__file__), "golden",
                                                          "obstacle_goldens.json")))}


def errors_line(levels):
    r = levels[-1]
    e1, ei, ae, _ = ob.report(r["m"], r["u"], r["F"])
    return "%.3e" % e1, "%.3e" % ei, "%.3f" % (100 * ae)


def test_golden_1_history_and_errors():
    """-da_refine 2 -ksp_rtol 1e-12 -snes_rtol 1e-10: the reduced-space Newton
    with (near) exact inner solves reproduces every printed number."""
    gold = GOLD[1]
    levels = ob.run(refine=2, rtol=1e-10)
    r = levels[0]
    assert r["m"] == gold["grid"][0] and r["its"] == gold["its"] and r["reason"] == 3
    assert ["%g" % f for f in r["fnorms"][:2]] == gold["snes_norms"][:2]
    assert r["fnorms"][2] < 1e-11
    assert errors_line(levels) == (gold["err1"], gold["errinf"], gold["area_err_pct"])


@pytest.mark.parametrize("test,refine,gs", [(2, 2, 0), (3, 0, 3), (4, 0, 2)])
def test_goldens_final_errors(test, refine, gs):
    """The discrete VI solution is unique: whatever the reference's linear
    solver or VI method (ASM/LU on 4 ranks, MG with grid sequencing, the
    semismooth method), its errors are the oracle's."""
    gold = GOLD[test]
    levels = ob.run(refine=refine, grid_sequence=gs)
    assert [levels[-1]["m"]] * 2 == gold["grid"]
    assert errors_line(levels) == (gold["err1"], gold["errinf"], gold["area_err_pct"])


def test_residual_is_the_fish_call_back_with_user_data():
    """The obstacle residual is Poisson2DFunctionLocal with f = 0 and g = the
    exact solution: the fish oracle (USER arrays) gives the same values."""
    m = 17
    h, X, Y = ob.coords(m)
    u = np.random.default_rng(2).standard_normal(m * m)
    g = np.ascontiguousarray(ob.u_exact(X, Y))
    f = np.zeros((m, m))
    gr = orc.grid(2, m, m, problem=orc.USER, L=(4.0, 4.0, 1.0))
    gr.f_user, gr.g_user = f.ctypes.data, g.ctypes.data
    F = orc.residual(gr, np.ascontiguousarray(u.reshape(1, m, m)))
    assert np.max(np.abs(F.ravel() - ob.residual(m, u))) <= 1e-13 * np.max(np.abs(F))
