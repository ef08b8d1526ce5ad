"""CPU tests of the oracle (the checker) against the reference's golden files
(c/ch6/output/fish.test1-8) and against independent restatements."""
import itertools
import json
import os

import numpy as np
import pytest

import _oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = json.load(open(os.path.join(HERE, "golden", "fish_goldens.json")))

# Which printed numbers of each regression run the restatement reproduces.
# Errors of runs at rtol 1e-12 (1, 7) equal the exact discrete solution's; runs
# 2, 5, 6, 8 use PETSc's one-rank default PC (ILU(0), natural ordering) which
# the oracle restates, so their rtol 1e-5 errors and run 6's iteration count
# are reproduced too.  Runs 3 and 4 use PETSc's SOR level smoother (and run 4
# two MPI ranks), which is not restated: only convergence is checked there.
PINNED_ERRORS = {1, 2, 5, 6, 7, 8}
PINNED_ITS = {6}


def half_ulp_of_print(s):
    """Half a unit in the last place of a %.3e string."""
    exp = int(s.split("e")[1])
    return 0.5 * 10.0 ** (exp - 3)


def parse(out):
    import re
    m = re.search(r"error \|u-uexact\|_inf = (\S+), \|u-uexact\|_h = (\S+)", out)
    r = {"errinf": m.group(1), "err2h": m.group(2)}
    m = re.search(r"iterations (\d+)", out)
    r["its"] = int(m.group(1)) if m else None
    m = re.search(r"0 SNES Function norm (\S+)", out)
    r["snes_norm0"] = m.group(1) if m else None
    m = re.search(r"problem (\S+) on (.*) grid:", out)
    r["problem"], r["grid"] = m.group(1), m.group(2)
    return r


@pytest.mark.parametrize("rec", GOLDEN, ids=lambda r: "fish.test%d" % r["test"])
def test_oracle_replays_golden(rec):
    out = orc.run_main(rec["args"])
    got = parse(out)
    assert got["problem"] == rec["problem"] and got["grid"] == rec["grid"]
    if rec["test"] in PINNED_ERRORS:
        _, full = orc.fish_solve(orc.options(rec["args"]))
        for key in ("errinf", "err2h"):
            # the full-precision value lies in the interval the printed %.3e
            # golden stands for (1D 5-point's exact error is 1/64, on a
            # rounding boundary, hence the 1e-9 relative slack)
            gold = float(rec[key])
            assert abs(full[key] - gold) <= half_ulp_of_print(rec[key]) + 1e-9 * gold, \
                (key, full[key], rec[key])
    else:
        assert float(got["errinf"]) < 5 * float(rec["errinf"])
    if rec["test"] in PINNED_ITS:
        assert got["its"] == rec["its"]
    if rec["snes_norm0"] is not None:
        assert got["snes_norm0"] == rec["snes_norm0"]
    if rec["its"] is not None:
        assert "converged due to CONVERGED_RTOL" in out


def dense_operator(g):
    """Assembled Jacobian of c/ch6/poissonfunctions.c:117-258 over all nodes."""
    shp = orc.shape(g)
    N = int(np.prod(shp))
    A = np.zeros((N, N))
    for n in range(N):
        e = np.zeros(N)
        e[n] = 1.0
        A[:, n] = orc.apply(g, e.reshape(shp)).ravel()
    return A


CASES = [
    (1, (9, 1, 1), (1.0, 1.0, 1.0), (1.0, 1.0, 1.0)),
    (2, (9, 5, 1), (1.0, 1.0, 1.0), (2.0, 0.5, 1.0)),
    (2, (7, 11, 1), (0.3, 2.0, 1.0), (1.0, 1.0, 1.0)),
    (3, (5, 7, 9), (0.01, 2.0, 100.0), (1.0, 1.0, 1.0)),
    (3, (5, 5, 5), (1.0, 1.0, 1.0), (1.0, 2.0, 3.0)),
]


@pytest.mark.parametrize("case", CASES)
def test_apply_is_symmetric_and_matches_linearised_residual(case):
    dim, m, c, L = case
    g = orc.grid(dim, *m, problem=orc.MANUPOLY, c=c, L=L)
    A = dense_operator(g)
    assert np.allclose(A, A.T, rtol=0, atol=1e-13 * np.abs(A).max())
    rng = np.random.default_rng(3)
    u = rng.standard_normal(orc.shape(g))
    p = rng.standard_normal(orc.shape(g))
    # F is affine: F(u + p) - F(u) = J p (boundary columns eliminated)
    lhs = orc.residual(g, u + p) - orc.residual(g, u)
    assert np.allclose(lhs, orc.apply(g, p), rtol=1e-12, atol=1e-12 * np.abs(lhs).max())


def residual_loop(g, u):
    """Independent pure-Python restatement of poissonfunctions.c:29-115 (2D/3D)."""
    h = [g.Lx / (g.mx - 1), g.Ly / (g.my - 1), g.Lz / (g.mz - 1) if g.dim == 3 else 1.0]
    vol = h[0] * h[1] * (h[2] if g.dim == 3 else 1.0)
    sc = [c * vol / hh ** 2 for c, hh in zip((g.cx, g.cy, g.cz), h)][: g.dim]
    diag = 2 * sum(sc)
    gf = lambda i, j, k: orc.lib().or_gfun(ctypes_grid(g), i * h[0], j * h[1], k * h[2])
    ff = lambda i, j, k: orc.lib().or_ffun(ctypes_grid(g), i * h[0], j * h[1], k * h[2])
    F = np.zeros_like(u)
    m = (g.mx, g.my, g.mz)
    for k, j, i in itertools.product(range(g.mz), range(g.my), range(g.mx)):
        idx = (i, j, k)
        if any(idx[d] in (0, m[d] - 1) for d in range(g.dim)):
            F[k, j, i] = (u[k, j, i] - gf(i, j, k)) * diag
            continue
        v = diag * u[k, j, i] - vol * ff(i, j, k)
        for d in range(g.dim):
            for s in (-1, 1):
                q = list(idx)
                q[d] += s
                nb = gf(*q) if q[d] in (0, m[d] - 1) else u[q[2], q[1], q[0]]
                v -= sc[d] * nb
        F[k, j, i] = v
    return F


def ctypes_grid(g):
    import ctypes
    orc.lib().or_gfun.argtypes = [ctypes.POINTER(orc.Grid)] + [ctypes.c_double] * 3
    orc.lib().or_gfun.restype = ctypes.c_double
    orc.lib().or_ffun.argtypes = [ctypes.POINTER(orc.Grid)] + [ctypes.c_double] * 3
    orc.lib().or_ffun.restype = ctypes.c_double
    return ctypes.byref(g)


@pytest.mark.parametrize("problem", [orc.MANUPOLY, orc.MANUEXP])
@pytest.mark.parametrize("dim,m", [(2, (6, 9, 1)), (3, (5, 6, 7))])
def test_residual_matches_loop_restatement(problem, dim, m):
    g = orc.grid(dim, *m, problem=problem)
    u = np.random.default_rng(1).standard_normal(orc.shape(g))
    assert np.allclose(orc.residual(g, u), residual_loop(g, u), rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("case", CASES)
def test_exact_solve_matches_dense_solve(case):
    dim, m, c, L = case
    g = orc.grid(dim, *m, problem=orc.ZERO, c=c, L=L)
    A = dense_operator(g)
    b = np.random.default_rng(7).standard_normal(orc.shape(g))
    x = orc.exact_solve(g, b)
    xd = np.linalg.solve(A, b.ravel()).reshape(b.shape)
    assert np.allclose(x, xd, rtol=1e-11, atol=1e-11 * np.abs(xd).max())


def test_restriction_is_transpose_of_prolongation():
    import ctypes
    for dim, mf in [(1, (17, 1, 1)), (2, (9, 17, 1)), (3, (9, 5, 17))]:
        gf = orc.grid(dim, *mf)
        mc = [(v - 1) // 2 + 1 if d < dim else 1 for d, v in enumerate(mf)]
        gc = orc.grid(dim, *mc)
        rng = np.random.default_rng(dim)
        r = rng.standard_normal(orc.shape(gf))
        xc = rng.standard_normal(orc.shape(gc))
        bc = np.empty(orc.shape(gc))
        orc.lib().or_restrict(ctypes.byref(gf), ctypes.byref(gc), r, bc)
        px = np.zeros(orc.shape(gf))
        orc.lib().or_prolong_add(ctypes.byref(gf), ctypes.byref(gc), xc, px)
        assert abs(np.vdot(bc, xc) - np.vdot(r, px)) < 1e-11 * abs(np.vdot(r, px))
        # P reproduces coarse-grid linear functions exactly (Q1)
        gcoords = np.meshgrid(*[np.linspace(0, 1, v) for v in reversed(mc)], indexing="ij")
        lin = 1.0 + sum((d + 2) * gcoords[d] for d in range(3))
        fine = np.zeros(orc.shape(gf))
        orc.lib().or_prolong_add(ctypes.byref(gf), ctypes.byref(gc), np.ascontiguousarray(lin), fine)
        fcoords = np.meshgrid(*[np.linspace(0, 1, v) for v in reversed(mf)], indexing="ij")
        flin = 1.0 + sum((d + 2) * fcoords[d] for d in range(3))
        assert np.allclose(fine, flin, atol=1e-13)


@pytest.mark.parametrize("args", [
    "-fsh_dim 2 -fsh_problem manupoly -da_refine 4 -pc_type mg -ksp_rtol 1e-13",
    "-fsh_dim 3 -fsh_problem manuexp -da_refine 3 -pc_type mg -ksp_rtol 1e-13",
    "-fsh_dim 3 -fsh_problem manupoly -da_refine 2 -pc_type mg -ksp_rtol 1e-13 -fsh_cx 0.5 -fsh_cy 2 -fsh_cz 3",
])
def test_tight_mg_solve_equals_exact_solve(args):
    o = orc.options(args)
    u, rep = orc.fish_solve(o)
    g = o.grid
    # exact discrete solution: u* = u0 - J^{-1} F(u0)
    u0 = orc.initial(g, 0, True)
    ustar = u0 - orc.exact_solve(g, orc.residual(g, u0))
    assert np.allclose(u, ustar, rtol=0, atol=1e-11 * np.abs(ustar).max())
    e_inf, e_h = orc.errnorms(g, ustar)
    assert abs(rep["errinf"] - e_inf) <= 1e-8 * e_inf
    assert rep["reason"] == 2


def test_mg_cycle_reduces_error_like_a_multigrid():
    # V(2,2) Chebyshev/Jacobi CG should need O(10) iterations independent of h
    its = []
    for r in (4, 5, 6):
        o = orc.options("-fsh_dim 2 -fsh_problem manupoly -pc_type mg -ksp_rtol 1e-10 -da_refine %d" % r)
        its.append(orc.fish_solve(o)[1]["its"])
    assert max(its) <= 14 and max(its) - min(its) <= 2, its


def test_oracle_is_deterministic_across_threads():
    import subprocess
    args = "-fsh_dim 3 -fsh_problem manupoly -da_refine 3 -pc_type mg -ksp_rtol 1e-10 -ksp_monitor".split()
    outs = []
    for nt in ("1", "4"):
        p = subprocess.run([orc.EXE] + args, stdout=subprocess.PIPE, text=True,
                           env=dict(os.environ, OMP_NUM_THREADS=nt))
        outs.append(p.stdout)
    assert outs[0] == outs[1]


@pytest.mark.parametrize("dim,m,c,L", [(2, (17, 9), (1.0, 0.5, 1.0), (1.0, 2.0, 1.0)),
                                       (3, (9, 17, 5), (1.0, 2.0, 0.3), (1.0, 1.0, 3.0)),
                                       (3, (33, 33, 33), (1.0, 1.0, 1.0), (1.0, 1.0, 1.0))])
def test_fft_exact_solve_equals_the_dense_sine_transform_solve(dim, m, c, L):
    """The FFT form of the exact solve (used for grids too large for the
    dense transforms) gives the dense form's solution to rounding."""
    g = orc.grid(dim, *m, problem=orc.ZERO, c=c, L=L)
    b = np.random.default_rng(dim).standard_normal(orc.shape(g))
    x1 = orc.exact_solve(g, b)
    x2 = orc.exact_solve_dst(g, b)
    assert np.max(np.abs(x1 - x2)) <= 1e-12 * np.max(np.abs(x1))
    # and it solves the system: the oracle's operator maps it back to b
    assert np.max(np.abs(orc.apply(g, x2) - b)) <= 1e-10 * np.max(np.abs(b))
