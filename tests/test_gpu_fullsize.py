"""GPU parity at the sizes the benchmark reports, against independent CPU
checks (the oracle's FP64 operators and an exact sine-transform solve of the
same discrete system), so that faults that appear only at large sizes --
index arithmetic past 2^31 elements, reductions over many blocks, level
shapes of deep hierarchies -- cannot pass unseen:

  * 3D 513^3 (the bench's -da_refine 8 workload), FP64 and mixed forms: the
    solution against the exact discrete solution, the reported error against
    the exact discrete solution's error (fish.c's error report,
    c/ch6/fish.c:254-280), and the true residual recomputed by the oracle;
  * a batch holding 513^2 and 257^2 instances: every instance's residual
    recomputed by the oracle and its solution against the exact solve;
  * the minimal-surface sequence to 1025^2 (c/ch7/minimal.c with grid
    sequencing): the oracle's FP64 residual of the final iterate;
  * served requests of 1025^2 (2D) and 257^3 (3D).

The solution tolerances follow from the stopping test: a true relative
residual rho bounds the relative algebraic error by kappa * rho (kappa of
the Jacobi-scaled operator, about 1e5 at 513^3 and 4e5 at 1025^2); the
bounds below sit between the measured errors and that worst case.
"""
import numpy as np
import pytest

import _oracle as orc

pytestmark = pytest.mark.gpu

BENCH3D = ("-fsh_dim 3 -fsh_problem manupoly -da_refine 8 -pc_type mg -mg_levels_ksp_type chebyshev "
           "-mg_levels_pc_type jacobi -ksp_rtol 1e-10 -ksp_norm_type unpreconditioned")


@pytest.fixture(scope="module")
def exact513():
    """The exact discrete solution of the 513^3 manupoly system and its errors."""
    o = orc.options(BENCH3D)
    g = o.grid
    u0 = orc.initial(g, 0, True)
    ustar = u0 - orc.exact_solve_dst(g, orc.residual(g, u0))
    return g, ustar, orc.errnorms(g, ustar)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_513cube_solution_is_the_exact_discrete_solution(cuda, exact513, prec):
    import torch
    import p4pdes_gb300 as fg
    g, ustar, (einf, e2h) = exact513
    o = fg.options(BENCH3D + " -fsh_precision " + prec)
    u = torch.empty(o.shape, dtype=torch.float64, device=cuda)
    with fg.Solver(o) as s:
        rep = s.solve(u)
    assert rep.reason == 2 and rep.true_rel_resid <= 1e-10
    uh = u.cpu().numpy()
    del u
    torch.cuda.empty_cache()
    scale = np.max(np.abs(ustar))
    err = np.max(np.abs(uh - ustar)) / scale
    F = orc.residual(g, uh)
    relres = np.linalg.norm(F) / rep.fnorm0
    print("\n513^3 %s: its %d outer %d, |u - u*|/|u*| = %.3e, oracle rel. residual %.3e (reported %.3e), "
          "errinf %.6e vs exact %.6e" % (prec, rep.its, rep.outer_its, err, relres, rep.true_rel_resid,
                                         rep.errinf, einf))
    assert err <= 1e-10   # measured 1.2e-12 (both forms)
    assert relres <= 1.2e-10
    # the reported discretisation error is the exact discrete solution's
    assert abs(rep.errinf - einf) <= 1e-5 * einf and abs(rep.err2h - e2h) <= 1e-5 * e2h


def test_batch_with_513_and_257_instances(cuda):
    import torch
    import p4pdes_gb300 as fg
    sizes = [513, 257, 129, 257, 513, 65, 33]
    rng = np.random.default_rng(11)
    fs = [rng.standard_normal((n, n)) for n in sizes]
    ft = [torch.from_numpy(f).cuda() for f in fs]
    ut = [torch.full_like(f, float("nan")) for f in ft]
    with fg.Batch(sizes, rtol=1e-8) as b:
        rep = b.solve(ft, ut)
        inner, outer, rel, reason = b.results()
    assert rep.converged == len(sizes)
    for q, (n, f, u) in enumerate(zip(sizes, fs, ut)):
        uh = u.cpu().numpy()
        g = orc.grid(2, n, n, problem=orc.ZERO)
        bb = f / (n - 1) ** 2
        bb[0, :] = bb[-1, :] = bb[:, 0] = bb[:, -1] = 0.0
        bb = np.ascontiguousarray(bb[None])
        r = bb - orc.apply(g, np.ascontiguousarray(uh[None]))
        relres = np.linalg.norm(r) / np.linalg.norm(bb)
        ustar = orc.exact_solve_dst(g, bb)[0]
        relerr = np.max(np.abs(uh - ustar)) / np.max(np.abs(ustar))
        print("batch n=%d: outer %d inner %d, oracle rel. residual %.3e (reported %.3e), rel. error %.3e"
              % (n, outer[q], inner[q], relres, rel[q], relerr))
        assert reason[q] == 2 and relres <= 1.2e-8 and abs(relres - rel[q]) <= 1e-3 * rel[q]
        assert relerr <= 1e-7  # measured <= 5e-10


def test_minimal_surface_1025_final_iterate(cuda):
    import p4pdes_gb300 as fg
    import _ms_oracle as ms
    o = fg.ms_options("-da_grid_x 33 -da_grid_y 33 -snes_grid_sequence 5 -snes_rtol 1e-10")
    u = np.empty((1025, 1025))
    with fg.MsSolver(o) as s:
        rep = s.solve(u)
    last = rep.ngrids - 1
    assert rep.m[last] == 1025 and all(rep.reason[k] > 0 for k in range(rep.ngrids))
    g = ms.grid(1025)
    fn = np.linalg.norm(ms.residual(g, u.ravel()))
    err = np.max(np.abs(u.ravel() - ms.exact(g).ravel()))
    print("\nminimal 1025^2: its %s, oracle |F| %.3e (reported %.3e, first %.3e), err %.4e (reported %.4e)"
          % ([rep.its[k] for k in range(rep.ngrids)], fn, rep.fnorm[last][rep.its[last]], rep.fnorm[last][0],
             err, rep.errinf))
    assert abs(fn - rep.fnorm[last][rep.its[last]]) <= 1e-3 * fn + 1e-14
    # PETSc's tests (SNESConvergedDefault): |F| <= rtol |F0| (CONVERGED_FNORM_RELATIVE, 3), or a
    # Newton step below stol |u| (CONVERGED_SNORM_RELATIVE, 4), after which |F| is at the level of
    # the step's square (measured 1.8e-10 |F0| on this grid)
    reason = rep.reason[last]
    assert reason in (3, 4)
    assert fn <= (1e-10 if reason == 3 else 1e-8) * rep.fnorm[last][0]
    assert abs(rep.errinf - err) <= 1e-9 + 1e-6 * err


@pytest.mark.parametrize("dim,n", [(2, 1025), (3, 257)])
def test_served_request_at_full_size(cuda, dim, n):
    import p4pdes_gb300 as fg
    f = np.random.default_rng(5).standard_normal((n,) * dim)
    u = np.full_like(f, np.nan)
    with fg.Server(workers=2) as srv:
        res = srv.wait(srv.submit(dim, n, f, u), 300000.0)
    assert res.status == 0
    g = orc.grid(dim, n, n, n, problem=orc.ZERO)
    b = f / (n - 1) ** dim
    for ax in range(dim):
        sl = [slice(None)] * dim
        sl[ax] = 0
        b[tuple(sl)] = 0.0
        sl[ax] = -1
        b[tuple(sl)] = 0.0
    shp = orc.shape(g)
    b = np.ascontiguousarray(b.reshape(shp))
    uh = np.ascontiguousarray(u.reshape(shp))
    relres = np.linalg.norm(b - orc.apply(g, uh)) / np.linalg.norm(b)
    ustar = orc.exact_solve_dst(g, b)
    relerr = np.max(np.abs(uh - ustar)) / np.max(np.abs(ustar))
    print("\nserved %dD n=%d: outer %d its %d, oracle rel. residual %.3e (reported %.3e), rel. error %.3e"
          % (dim, n, res.outer_its, res.its, relres, res.rel_resid, relerr))
    assert relres <= 1.2e-8 and abs(relres - res.rel_resid) <= 1e-3 * res.rel_resid
    assert relerr <= 1e-7  # measured 2.7e-10 (2D), 2.2e-9 (3D)
