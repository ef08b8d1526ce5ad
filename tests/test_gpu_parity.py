"""GPU parity tests: libfishgpu.so (through its C ABI) against the CPU oracle.

Tolerances (FP64 form): call-back outputs agree to 1e-13 relative (same
formulas, different FMA contraction and exp() implementation); the CG residual
history agrees to 1e-8 relative per iteration and the iteration count and
reason agree exactly; discretisation errors agree to 1e-9 relative.
Mixed form: final error within 1.01x of the FP64 error, true relative residual
below rtol.
"""
import json
import os
import re
import subprocess

import numpy as np
import pytest

import _oracle as orc

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = json.load(open(os.path.join(ROOT, "tests", "golden", "fish_goldens.json")))


def fgmod():
    import p4pdes_gb300 as fg
    return fg


def info_ctx(g, xs=None, xm=None):
    fg = fgmod()
    inf = fg.Info()
    inf.dim, inf.mx, inf.my, inf.mz = g.dim, g.mx, g.my, g.mz
    s = xs or (0, 0, 0)
    w = xm or (g.mx, g.my, g.mz)
    inf.xs, inf.ys, inf.zs = s
    inf.xm, inf.ym, inf.zm = w
    inf.xmax[0], inf.xmax[1], inf.xmax[2] = g.Lx, g.Ly, g.Lz
    c = fg.Ctx()
    c.Lx, c.Ly, c.Lz, c.cx, c.cy, c.cz = g.Lx, g.Ly, g.Lz, g.cx, g.cy, g.cz
    c.problem, c.dim = g.problem, g.dim
    return inf, c


def tcuda(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


GRIDS = [
    (1, (17, 1, 1), orc.MANUPOLY, (1.0, 1.0, 1.0), (1.0, 1.0, 1.0)),
    (1, (9, 1, 1), orc.MANUEXP, (1.0, 1.0, 1.0), (2.0, 1.0, 1.0)),
    (2, (33, 17, 1), orc.MANUPOLY, (0.3, 2.0, 1.0), (1.0, 1.0, 1.0)),
    (2, (65, 65, 1), orc.MANUEXP, (1.0, 1.0, 1.0), (1.0, 2.0, 1.0)),
    (2, (37, 3, 1), orc.MANUPOLY, (1.0, 1.0, 1.0), (1.0, 1.0, 1.0)),
    (3, (9, 9, 9), orc.MANUPOLY, (0.01, 2.0, 100.0), (1.0, 1.0, 1.0)),
    (3, (33, 17, 65), orc.MANUEXP, (1.0, 1.0, 1.0), (1.0, 1.0, 1.0)),
    (3, (35, 6, 5), orc.MANUPOLY, (1.0, 1.5, 0.5), (1.0, 0.5, 3.0)),
]


@pytest.mark.parametrize("case", GRIDS)
def test_residual_callback_matches_oracle(cuda, case):
    import torch
    fg = fgmod()
    dim, m, prob, c, L = case
    g = orc.grid(dim, *m, problem=prob, c=c, L=L)
    u = np.random.default_rng(11).standard_normal(orc.shape(g))
    ref = orc.residual(g, u)
    inf, ctx = info_ctx(g)
    F = torch.full(orc.shape(g), np.nan, dtype=torch.float64, device=cuda)
    getattr(fg, "Poisson%dDFunctionLocal" % dim)(inf, tcuda(u), F, ctx)
    torch.cuda.synchronize()
    got = F.cpu().numpy()
    assert np.max(np.abs(got - ref)) <= 1e-13 * np.max(np.abs(ref))


@pytest.mark.parametrize("case", GRIDS)
def test_apply_and_dot_match_oracle(cuda, case):
    import torch
    fg = fgmod()
    dim, m, prob, c, L = case
    g = orc.grid(dim, *m, problem=prob, c=c, L=L)
    p = np.random.default_rng(5).standard_normal(orc.shape(g))
    ref = orc.apply(g, p)
    inf, ctx = info_ctx(g)
    q = torch.empty(orc.shape(g), dtype=torch.float64, device=cuda)
    d = getattr(fg, "Poisson%dDOperatorApply" % dim)(inf, tcuda(p), q, ctx)
    torch.cuda.synchronize()
    assert np.max(np.abs(q.cpu().numpy() - ref)) <= 1e-13 * np.max(np.abs(ref))
    dref = float(np.vdot(p, ref))
    assert abs(d.item() - dref) <= 1e-12 * abs(dref)


def test_callbacks_respect_the_owned_range(cuda):
    import torch
    fg = fgmod()
    g = orc.grid(3, 17, 13, 11, problem=orc.MANUPOLY, c=(1.0, 2.0, 3.0))
    u = np.random.default_rng(2).standard_normal(orc.shape(g))
    ref = orc.residual(g, u)
    inf, ctx = info_ctx(g, xs=(3, 1, 4), xm=(9, 10, 5))
    F = torch.full(orc.shape(g), -7.0, dtype=torch.float64, device=cuda)
    fg.Poisson3DFunctionLocal(inf, tcuda(u), F, ctx)
    got = F.cpu().numpy()
    box = (slice(4, 9), slice(1, 11), slice(3, 12))
    assert np.max(np.abs(got[box] - ref[box])) <= 1e-13 * np.max(np.abs(ref))
    mask = np.ones_like(got, dtype=bool)
    mask[box] = False
    assert np.all(got[mask] == -7.0)
    # empty owned range is a no-op
    inf.xm = 0
    fg.Poisson3DFunctionLocal(inf, tcuda(u), F, ctx)
    assert np.all(F.cpu().numpy()[mask] == -7.0)


def test_user_arrays_match_builtin_problem(cuda):
    """FISHGPU_USER with f and g sampled from manupoly gives the built-in result."""
    import torch
    fg = fgmod()
    g = orc.grid(2, 33, 17, problem=orc.MANUPOLY)
    h = [g.Lx / (g.mx - 1), g.Ly / (g.my - 1)]
    jj, ii = np.meshgrid(np.arange(g.my), np.arange(g.mx), indexing="ij")
    x, y = ii * h[0], jj * h[1]
    gv = (x * x * (1 - x * x) * y * y * (y * y - 1))[None]
    fv = -((2 * (1 - 6 * x * x)) * (y * y * (y * y - 1)) + (x * x * (1 - x * x)) * (2 * (6 * y * y - 1)))[None]
    u = np.random.default_rng(9).standard_normal(orc.shape(g))
    inf, ctx = info_ctx(g)
    F1 = torch.empty(orc.shape(g), dtype=torch.float64, device=cuda)
    fg.Poisson2DFunctionLocal(inf, tcuda(u), F1, ctx)
    ft, gt = tcuda(fv), tcuda(gv)
    ctx.problem, ctx.f, ctx.g = fg.USER, ft.data_ptr(), gt.data_ptr()
    F2 = torch.empty_like(F1)
    fg.Poisson2DFunctionLocal(inf, tcuda(u), F2, ctx)
    assert torch.allclose(F1, F2, rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("dim,m", [(1, (33, 1, 1)), (2, (17, 9, 1)), (3, (9, 17, 5))])
@pytest.mark.parametrize("itype,gb", [(0, True), (0, False), (1, True), (1, False)])
def test_initial_state_and_exact_match_oracle(cuda, dim, m, itype, gb):
    import torch
    fg = fgmod()
    g = orc.grid(dim, *m, problem=orc.MANUEXP)
    inf, ctx = info_ctx(g)
    u = torch.empty(orc.shape(g), dtype=torch.float64, device=cuda)
    fg.InitialState(inf, itype, gb, u, ctx, seed=1234)
    ref = orc.initial(g, itype, gb, seed=1234)
    got = u.cpu().numpy()
    # same generator (splitmix64 of the dense index) on both sides
    assert np.max(np.abs(got - ref)) <= 1e-14 * max(1.0, np.max(np.abs(ref)))
    fg.FormUExact(inf, u, ctx)
    assert np.max(np.abs(u.cpu().numpy() - orc.exact(g))) <= 1e-14 * np.max(np.abs(orc.exact(g)))
    e = fg.error_norms(inf, tcuda(ref), ctx)
    eref = orc.errnorms(g, ref)
    assert abs(e[0] - eref[0]) <= 1e-14 * eref[0] and abs(e[1] - eref[1]) <= 1e-12 * eref[1]


# ---------------------------------------------------------------- solver parity
SOLVES = [r["args"] + ["-pc_type", "mg"] for r in GOLDEN] + [
    "-fsh_dim 2 -fsh_problem manupoly -da_refine 7 -pc_type mg -mg_levels_ksp_type chebyshev "
    "-mg_levels_pc_type jacobi -ksp_rtol 1e-10".split(),
    "-fsh_dim 3 -fsh_problem manupoly -da_refine 5 -pc_type mg -ksp_rtol 1e-10".split(),
    "-fsh_dim 3 -fsh_problem manuexp -da_refine 4 -pc_type mg -ksp_rtol 1e-10 -ksp_norm_type unpreconditioned".split(),
    "-fsh_dim 2 -fsh_problem manupoly -da_refine 5 -pc_type mg -pc_mg_levels 3 -ksp_rtol 1e-10".split(),
    "-fsh_dim 3 -fsh_problem manupoly -da_refine 4 -pc_type mg -pc_mg_levels 2 -ksp_rtol 1e-9".split(),
    "-fsh_dim 2 -fsh_problem manupoly -da_refine 5 -pc_type mg -mg_levels_ksp_max_it 3 -ksp_rtol 1e-10".split(),
    "-fsh_dim 2 -fsh_problem manupoly -da_refine 4 -pc_type mg -pc_mg_cycle_type w -ksp_rtol 1e-10".split(),
    "-fsh_dim 2 -fsh_problem manupoly -da_refine 4 -pc_type mg -mg_levels_ksp_type richardson "
    "-mg_levels_ksp_richardson_scale 0.6 -mg_levels_ksp_max_it 2 -ksp_rtol 1e-8".split(),
    "-fsh_dim 2 -fsh_problem manupoly -da_refine 4 -pc_type jacobi -ksp_rtol 1e-8".split(),
    "-fsh_dim 2 -fsh_problem manupoly -da_refine 3 -pc_type none -ksp_rtol 1e-8".split(),
    "-fsh_dim 3 -fsh_problem manupoly -da_refine 3 -pc_type mg -fsh_initial_type random -fsh_seed 77 -ksp_rtol 1e-10".split(),
    "-fsh_dim 2 -fsh_problem manupoly -da_grid_x 5 -da_grid_y 3 -da_refine 4 -fsh_Lx 2 -fsh_cy 3 -pc_type mg -ksp_rtol 1e-10".split(),
    "-fsh_dim 3 -fsh_problem manupoly -da_refine 3 -pc_type mg -mg_levels_ksp_chebyshev_esteig 0,0.2,0,1.2 -ksp_rtol 1e-10".split(),
]


def compare_runs(args, fg_rep, ref):
    assert fg_rep.reason == ref["reason"], args
    assert fg_rep.its == ref["its"], (fg_rep.its, ref["its"], args)
    h = fg_rep.history()
    assert len(h) == len(ref["hist"])
    # 1e-8 relative per iteration; entries at round-off level (below 1e-13 of
    # the initial norm, e.g. after an exact coarse solve) are rounding noise
    floor = 1e-13 * ref["hist"][0]
    for a, b in zip(h, ref["hist"]):
        assert abs(a - b) <= 1e-8 * abs(b) + floor, (a, b, args)
    assert abs(fg_rep.fnorm0 - ref["fnorm0"]) <= 1e-12 * ref["fnorm0"]
    for key in ("errinf", "err2h"):
        assert abs(getattr(fg_rep, key) - ref[key]) <= 1e-9 * ref[key] + 1e-15, (key, args)


@pytest.mark.parametrize("args", SOLVES, ids=lambda a: " ".join(a)[:90])
def test_fp64_solve_matches_oracle(cuda, args):
    fg = fgmod()
    o = fg.options(args)
    u, rep = fg.solve(o)
    oo = orc.options(args)
    uref, ref = orc.fish_solve(oo)
    compare_runs(args, rep, ref)
    diff = np.max(np.abs(u.cpu().numpy() - uref))
    assert diff <= 1e-9 * max(1e-300, np.max(np.abs(uref)))


def test_fp64_solve_reaches_the_exact_discrete_solution(cuda):
    fg = fgmod()
    args = "-fsh_dim 3 -fsh_problem manupoly -da_refine 6 -pc_type mg -ksp_rtol 1e-13"
    u, rep = fg.solve(fg.options(args))
    g = orc.options(args).grid
    u0 = orc.initial(g, 0, True)
    ustar = u0 - orc.exact_solve(g, orc.residual(g, u0))
    assert np.max(np.abs(u.cpu().numpy() - ustar)) <= 1e-11 * np.max(np.abs(ustar))
    e = orc.errnorms(g, ustar)
    assert abs(rep.errinf - e[0]) <= 1e-8 * e[0]


@pytest.mark.parametrize("args", [
    "-fsh_dim 2 -fsh_problem manupoly -da_refine 7 -pc_type mg -ksp_rtol 1e-10",
    "-fsh_dim 3 -fsh_problem manupoly -da_refine 5 -pc_type mg -ksp_rtol 1e-10",
    "-fsh_dim 3 -fsh_problem manuexp -da_refine 4 -pc_type mg -ksp_rtol 1e-10",
])
def test_mixed_form_matches_fp64_error(cuda, args):
    fg = fgmod()
    _, r64 = fg.solve(fg.options(args + " -ksp_norm_type unpreconditioned"))
    _, rmx = fg.solve(fg.options(args + " -fsh_precision mixed"))
    assert rmx.reason == 2 and rmx.outer_its >= 1
    assert rmx.true_rel_resid <= 1e-10
    assert rmx.errinf <= 1.01 * r64.errinf and rmx.err2h <= 1.01 * r64.err2h
    # the FP64 outer history is the true residual and decreases
    h = rmx.history()
    assert all(b < a for a, b in zip(h, h[1:]))


def test_mixed_form_inner_iterations_do_not_depend_on_the_outer_norm_option(cuda):
    """The inner FP32 CG always stops on its own unpreconditioned residual,
    whatever -ksp_norm_type says (that option governs the FP64 form)."""
    fg = fgmod()
    base = "-fsh_dim 3 -fsh_problem manupoly -da_refine 5 -pc_type mg -ksp_rtol 1e-10 -fsh_precision mixed"
    _, a = fg.solve(fg.options(base))
    _, b = fg.solve(fg.options(base + " -ksp_norm_type unpreconditioned"))
    assert a.its == b.its and a.outer_its == b.outer_its and a.its <= 30
    assert a.history() == b.history()


@pytest.mark.parametrize("args", [
    "-fsh_dim 3 -fsh_problem manupoly -da_refine 5 -pc_type mg -ksp_rtol 1e-10",
    "-fsh_dim 3 -fsh_problem manuexp -da_grid_x 5 -da_grid_y 3 -da_grid_z 9 -da_refine 5 -pc_type mg -ksp_rtol 1e-10",
    "-fsh_dim 3 -fsh_problem manupoly -da_refine 6 -pc_mg_levels 4 -fsh_cx 0.5 -fsh_cz 2 -ksp_rtol 1e-10",
])
def test_fused_post_smoother_matches_two_steps(cuda, args):
    """The temporally blocked post-smoother computes every point with the
    operations of the two separate Chebyshev steps: same iteration counts,
    the same solution to FP32 rounding of the fused dot products."""
    fg = fgmod()
    # the launch-per-phase solve (the persistent one has no fused post-smoother)
    u1, a = fg.solve(fg.options(args + " -fsh_precision mixed -fsh_fuse_smooth 1 -fsh_persist 0"))
    u0, b = fg.solve(fg.options(args + " -fsh_precision mixed -fsh_fuse_smooth 0 -fsh_persist 0"))
    assert a.reason == b.reason == 2 and a.its == b.its and a.outer_its == b.outer_its
    h0 = b.history()[0]
    assert a.history()[0] == h0  # the FP64 residual before any V-cycle
    for x, y in zip(a.history(), b.history()):  # later steps carry FP32 rounding of the inner solves
        assert abs(x - y) <= 1e-2 * abs(y) + 1e-13 * h0
    d = (u1 - u0).abs().max().item() / u0.abs().max().item()
    assert d <= 1e-9, d
    assert abs(a.errinf - b.errinf) <= 1e-6 * b.errinf


def test_zero_problem_converges_at_iteration_zero(cuda):
    fg = fgmod()
    u, rep = fg.solve(fg.options("-fsh_dim 2 -fsh_problem zero -da_refine 3 -pc_type mg"))
    assert rep.its == 0 and rep.reason == 3 and rep.errinf == 0.0


def test_iteration_cap_reports_not_converged(cuda):
    import torch
    fg = fgmod()
    o = fg.options("-fsh_dim 2 -fsh_problem manupoly -da_refine 5 -pc_type jacobi -ksp_max_it 3 -ksp_rtol 1e-12")
    u = torch.empty(o.shape, dtype=torch.float64, device=cuda)
    with fg.Solver(o) as s:
        rep = s.solve(u)
    assert rep.reason == -3 and rep.its == 3
    oo = orc.options("-fsh_dim 2 -fsh_problem manupoly -da_refine 5 -pc_type jacobi -ksp_max_it 3 -ksp_rtol 1e-12")
    assert orc.fish_solve(oo)[1]["its"] == 3


def test_nonfinite_user_data_is_reported(cuda):
    import torch
    fg = fgmod()
    o = fg.options("-fsh_dim 2 -da_refine 3 -pc_type mg")
    f = torch.zeros(o.shape, dtype=torch.float64, device=cuda)
    g = torch.zeros_like(f)
    f[0, 5, 5] = float("nan")
    o.ctx.problem, o.ctx.f, o.ctx.g = fg.USER, f.data_ptr(), g.data_ptr()
    u = torch.empty_like(f)
    with fg.Solver(o) as s:
        with pytest.raises(fg.FishError) as e:
            s.solve(u)
    assert e.value.code == 5


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
@pytest.mark.parametrize("args", [
    "-fsh_dim 3 -fsh_problem manupoly -da_refine 4 -pc_type mg -ksp_rtol 1e-10",
    "-fsh_dim 3 -fsh_problem manuexp -da_grid_x 5 -da_grid_y 3 -da_grid_z 9 -da_refine 3 -pc_type mg -ksp_rtol 1e-10",
    "-fsh_dim 2 -fsh_problem manupoly -da_refine 6 -pc_type mg -fsh_cx 0.5 -ksp_rtol 1e-10",
    "-fsh_dim 1 -fsh_problem manupoly -da_refine 6 -pc_type mg -ksp_rtol 1e-10",
])
def test_zero_initial_residual_matches_the_stencil(cuda, args, prec):
    """The initial residual from the zero initial state is a pointwise pass
    (interior rows of the Jacobian do not see boundary columns); the same u0
    given explicitly takes the FP64 stencil.  Histories and solutions agree to
    the bit."""
    import torch
    fg = fgmod()
    oa = fg.options(args + " -fsh_precision " + prec)
    ob = fg.options(args + " -fsh_precision " + prec)
    ob.initial_type = fg.INITIAL_GIVEN
    u0 = torch.empty(oa.shape, dtype=torch.float64, device=cuda)
    fg.InitialState(fg.info_for(oa), fg.INITIAL_ZEROS, 1, u0, oa.ctx)
    ua, ub = torch.empty_like(u0), u0.clone()
    with fg.Solver(oa) as s:
        ra = s.solve(ua)
    with fg.Solver(ob) as s:
        rb = s.solve(ub)
    assert ra.reason == rb.reason == 2 and ra.its == rb.its
    assert ra.history() == rb.history() and ra.fnorm0 == rb.fnorm0
    assert torch.equal(ua, ub)


@pytest.mark.parametrize("args", [
    "-fsh_dim 3 -fsh_problem manupoly -da_refine 4 -pc_type mg -ksp_rtol 1e-10 -fsh_precision mixed",
    "-fsh_dim 3 -fsh_problem manuexp -da_refine 4 -pc_type mg -ksp_rtol 1e-10",
    "-fsh_dim 2 -fsh_problem manupoly -da_refine 5 -pc_type mg -ksp_rtol 1e-10 -fsh_graph_iters 6",
])
def test_device_loop_matches_host_loop(cuda, args):
    """The CG loop as a conditional graph node (one launch per inner solve)
    runs the same kernels as the host-polled graphs: identical histories and
    solutions."""
    fg = fgmod()
    u1, a = fg.solve(fg.options(args + " -fsh_device_loop 1 -fsh_persist 0"))
    u0, b = fg.solve(fg.options(args + " -fsh_device_loop 0 -fsh_persist 0"))
    assert a.reason == b.reason == 2 and a.its == b.its and a.outer_its == b.outer_its
    assert a.history() == b.history()
    import torch
    assert torch.equal(u1, u0)


@pytest.mark.parametrize("args,gb", [
    ("-fsh_dim 3 -da_grid_x 5 -da_grid_y 3 -da_grid_z 9 -da_refine 3 -pc_type mg -ksp_rtol 1e-10", 1),
    ("-fsh_dim 2 -fsh_problem manupoly -da_refine 6 -pc_type mg -ksp_rtol 1e-10 -fsh_cx 0.5", 1),
    ("-fsh_dim 2 -da_refine 5 -pc_type mg -ksp_rtol 1e-10 -fsh_initial_gonboundary false", 0),
    ("-fsh_dim 1 -da_refine 7 -pc_type mg -ksp_rtol 1e-10", 1),
])
def test_user_data_start_matches_the_three_kernels(cuda, args, gb):
    """A mixed solve of user f and g from the zero state starts with one fused
    pass (u0, b = -F(u0), its norm); the same u0 given explicitly takes the
    initial-state, beff and stencil-residual kernels.  Histories and solutions
    agree to the bit."""
    import torch
    fg = fgmod()
    oa = fg.options(args + " -fsh_precision mixed")
    ob = fg.options(args + " -fsh_precision mixed")
    rng = np.random.default_rng(5)
    f = torch.from_numpy(rng.standard_normal(tuple(oa.shape))).to(cuda)
    gd = torch.from_numpy(rng.standard_normal(tuple(oa.shape))).to(cuda)
    for o in (oa, ob):
        o.ctx.problem, o.ctx.f, o.ctx.g = fg.USER, f.data_ptr(), gd.data_ptr()
    ob.initial_type = fg.INITIAL_GIVEN
    u0 = torch.empty(oa.shape, dtype=torch.float64, device=cuda)
    fg.InitialState(fg.info_for(oa), fg.INITIAL_ZEROS, gb, u0, oa.ctx)
    ua, ub = torch.empty_like(u0), u0.clone()
    with fg.Solver(oa) as s:
        ra = s.solve(ua)
    with fg.Solver(ob) as s:
        rb = s.solve(ub)
    assert ra.reason == rb.reason == 2 and ra.its == rb.its and ra.outer_its == rb.outer_its
    assert ra.history() == rb.history() and ra.fnorm0 == rb.fnorm0
    assert torch.equal(ua, ub)


def test_fp64_fma_rate_is_plausible(cuda):
    """The FP64 FMA probe used as the FP64 residual's roofline denominator:
    GB300's FP64 rate is ~1.2 TFLOP/s nominal, far below its FP32 rate."""
    fg = fgmod()
    t = fg.fp64_fma_rate(3)
    assert 0.3 < t < 5.0, t


def test_solver_is_reusable_and_deterministic(cuda):
    import torch
    fg = fgmod()
    o = fg.options("-fsh_dim 3 -fsh_problem manupoly -da_refine 4 -pc_type mg -ksp_rtol 1e-10")
    with fg.Solver(o) as s:
        u1 = torch.empty(o.shape, dtype=torch.float64, device=cuda)
        u2 = torch.empty_like(u1)
        r1 = s.solve(u1)
        r2 = s.solve(u2)
    assert torch.equal(u1, u2) and r1.history() == r2.history()


def test_host_array_entry_point(cuda):
    import ctypes
    fg = fgmod()
    o = fg.options("-fsh_dim 2 -fsh_problem manupoly -da_refine 5 -pc_type mg -ksp_rtol 1e-10")
    u = np.empty(o.shape)
    rep = fg.Report()
    rc = fg.load().fishgpu_solve_host(ctypes.byref(o), None, None, u.ctypes.data, ctypes.byref(rep))
    assert rc == 0
    uref, ref = orc.fish_solve(orc.options("-fsh_dim 2 -fsh_problem manupoly -da_refine 5 -pc_type mg -ksp_rtol 1e-10"))
    assert np.max(np.abs(u - uref)) <= 1e-9 * np.max(np.abs(uref))


@pytest.mark.parametrize("dim,refine", [(3, 4), (2, 6), (1, 6)])
def test_pinned_boundary_gather_equals_full_copy(cuda, dim, refine):
    """A pinned host g is read on the boundary only (gathered in place); the
    result is bit-identical to copying a pageable g whole, whatever g holds
    inside (the solver reads it nowhere else)."""
    import torch
    fg = fgmod()
    o = fg.options("-fsh_dim %d -da_refine %d -pc_type mg -ksp_rtol 1e-10 -fsh_precision mixed" % (dim, refine))
    o.ctx.problem = fg.USER
    rng = np.random.default_rng(9)
    f = rng.standard_normal(o.shape)
    g = rng.standard_normal(o.shape)
    g_inner_junk = g.copy()
    sl = tuple(slice(1, -1) if n > 1 else slice(None) for n in o.shape)
    g_inner_junk[sl] = 1e300
    u1, u2 = np.empty(o.shape), np.empty(o.shape)
    with fg.Solver(o) as s:
        s.solve_host(f, g, u1)                                   # pageable: copied whole
        gp = torch.from_numpy(g_inner_junk).pin_memory()
        r2 = s.solve_host(f, gp, u2)                             # pinned: boundary gather
        nb = s.host_bytes_in(gp) - 8 * f.size
        assert nb < 8 * g.size or dim == 1
        assert s.host_bytes_in(g) == 16 * f.size
    assert np.array_equal(u1, u2) and r2.reason > 0


@pytest.mark.parametrize("args", [
    "-fsh_dim 3 -da_refine 5 -pc_type mg -ksp_rtol 1e-10 -fsh_precision mixed",
    "-fsh_dim 2 -da_refine 7 -pc_type mg -ksp_rtol 1e-10",
    "-fsh_dim 3 -da_refine 4 -pc_type mg -ksp_rtol 1e-10 -fsh_precision mixed -fsh_persist 0",
])
def test_pipelined_host_solves_equal_single_calls(cuda, args):
    """fishgpu_solver_solve_host_many (the next f in and the last u out on
    copy streams while a problem is solved) gives every problem the solution,
    bit for bit, and the report of its own fishgpu_solver_solve_host call:
    different f and g per problem, pinned and pageable arrays, a NULL g."""
    import torch
    fg = fgmod()
    o = fg.options(args)
    o.ctx.problem = fg.USER
    rng = np.random.default_rng(21)
    n = 4
    fs = [rng.standard_normal(o.shape) for _ in range(n)]
    gs = [rng.standard_normal(o.shape) for _ in range(n - 1)] + [None]
    pin = [torch.from_numpy(f).pin_memory() for f in fs[:2]] + fs[2:]
    us = [torch.empty(o.shape, dtype=torch.float64).pin_memory(), np.empty(o.shape),
          torch.empty(o.shape, dtype=torch.float64).pin_memory(), np.empty(o.shape)]
    want = [np.empty(o.shape) for _ in range(n)]
    with fg.Solver(o) as s:
        ref = [s.solve_host(fs[k], gs[k], want[k]) for k in range(n)]
        reps = s.solve_host_many(pin, gs, us)
        u_zero_g = np.empty(o.shape)
        reps2 = s.solve_host_many(pin[:1], None, [u_zero_g])  # again, one problem, zero g
    for k in range(n):
        got = us[k].numpy() if hasattr(us[k], "numpy") else us[k]
        assert np.array_equal(got, want[k])
        assert reps[k].reason == ref[k].reason > 0 and reps[k].its == ref[k].its
        assert reps[k].outer_its == ref[k].outer_its
    assert reps2[0].reason > 0


@pytest.mark.parametrize("rec", [r for r in GOLDEN if r["test"] in (1, 7)],
                         ids=lambda r: "fish.test%d" % r["test"])
def test_fish_driver_replays_golden(cuda, rec):
    """The C driver with the reference's flags prints the reference's error
    line and SNES norm lines for the runs solved to rtol 1e-12 (runs that
    stop at rtol 1e-5 depend on PETSc's default ILU preconditioner, which the
    GPU library replaces by multigrid; the oracle pins those)."""
    exe = os.path.join(ROOT, "p4pdes_gb300", "bin", "fish")
    p = subprocess.run([exe] + rec["args"], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert p.returncode == 0, p.stderr
    want = [l for l in rec["stdout"].splitlines() if "error |u-uexact|" in l or "SNES Function norm" in l
            or l.startswith("problem ")]
    got = [l for l in p.stdout.splitlines() if "error |u-uexact|" in l or "SNES Function norm" in l
           or l.startswith("problem ")]
    assert got == want


def test_accurate_inner_form_needs_fewer_refinement_steps(cuda):
    """The accurate inner form (difference-form FP32 apply, inner solution
    accumulated in FP64) lifts the FP32 floor of the first refinement step
    from ~kappa 2^-24 to ~kappa pi h 2^-24: at 257^3 its first step reaches a
    true residual below what the standard form's can, so the solve needs
    fewer FP64 residuals; both forms keep the FP64 form's error."""
    fg = fgmod()
    base = ("-fsh_dim 3 -fsh_problem manupoly -da_refine 7 -pc_type mg -ksp_rtol 1e-10 "
            "-ksp_norm_type unpreconditioned")
    _, r64 = fg.solve(fg.options(base))
    _, std = fg.solve(fg.options(base + " -fsh_precision mixed -fsh_inner_accurate 0"))
    _, acc = fg.solve(fg.options(base + " -fsh_precision mixed -fsh_inner_accurate 1"))
    # a first inner solve asked for 3e-6 of kappa pi h 2^-24 (~2e-6 here): the accurate form gets there
    _, deep = fg.solve(fg.options(base + " -fsh_precision mixed -fsh_inner_accurate 1 -fsh_first_floor 0.1"))
    for r in (std, acc, deep):
        assert r.reason == 2 and r.true_rel_resid <= 1e-10
        assert r.errinf <= 1.01 * r64.errinf and r.err2h <= 1.01 * r64.err2h
    h_std, h_deep = std.history(), deep.history()
    assert h_std[1] / h_std[0] > 1e-4   # the standard form's first step stops at its floor, ~kappa 2^-24
    assert h_deep[1] / h_deep[0] < 1e-5  # measured 3.3e-7
    assert acc.outer_its == 2 and std.outer_its == 3


@pytest.mark.parametrize("args", [
    "-fsh_dim 3 -fsh_problem manupoly -da_refine 5 -pc_type mg -ksp_rtol 1e-10",
    "-fsh_dim 3 -fsh_problem manupoly -da_refine 5 -pc_type mg -ksp_rtol 1e-10 -fsh_precision mixed",
    "-fsh_dim 3 -fsh_problem manupoly -da_grid_x 5 -da_grid_y 3 -da_grid_z 9 -da_refine 4 -pc_type mg "
    "-ksp_rtol 1e-10 -fsh_cz 3",
    "-fsh_dim 3 -da_grid_x 9 -da_grid_y 17 -da_grid_z 5 -da_refine 3 -pc_type mg -ksp_rtol 1e-10 "
    "-fsh_precision mixed -pc_mg_cycle_type w",
    "-fsh_dim 3 -fsh_problem manuexp -da_refine 6 -pc_type mg -ksp_rtol 1e-10 -fsh_precision mixed",
])
def test_fused_residual_restriction_is_bit_identical(cuda, args):
    """The 3D levels' fused residual + restriction (v_resid_restrict) computes
    every fine residual and weighted sum as v_resid and v_restrict do, in the
    same order: the whole solve is identical to the two-kernel form, bit for
    bit (tile edges in x, y and z, odd level shapes, W-cycles)."""
    import torch
    fg = fgmod()
    u1, a = fg.solve(fg.options(args + " -fsh_fuse_restrict 1 -fsh_persist 0"))
    u0, b = fg.solve(fg.options(args + " -fsh_fuse_restrict 0 -fsh_persist 0"))
    assert a.reason == b.reason == 2 and a.its == b.its and a.outer_its == b.outer_its
    assert a.history() == b.history()
    assert torch.equal(u1, u0)


@pytest.mark.parametrize("args", [
    "-fsh_dim 3 -fsh_problem manupoly -da_refine 7 -pc_type mg -ksp_rtol 1e-10 -fsh_precision mixed",
    "-fsh_dim 3 -fsh_problem manupoly -da_grid_x 9 -da_grid_y 5 -da_grid_z 3 -da_refine 5 -pc_type mg "
    "-ksp_rtol 1e-10 -fsh_precision mixed -fsh_cz 2",
    "-fsh_dim 3 -fsh_problem manuexp -da_grid_x 5 -da_grid_y 9 -da_grid_z 17 -da_refine 6 -pc_type mg "
    "-ksp_rtol 1e-12 -fsh_precision mixed -fsh_inner_accurate 1",
])
def test_tma_apply_matches_the_slot_march(cuda, args):
    """The accurate CG update + apply fed by the TMA ring computes every p, w
    and y64 value as the slot-march kernel does; only p.w is summed in
    another order, so the solves agree to rounding: same iterations, both
    meet rtol, solutions agree to 1e-9 relative (tile edges in x, y and z at
    uneven grid shapes, first iteration, fresh and accumulated y64)."""
    fg = fgmod()
    u1, a = fg.solve(fg.options(args + " -fsh_tma_apply 1 -fsh_persist 0"))
    u0, b = fg.solve(fg.options(args + " -fsh_tma_apply 0 -fsh_persist 0"))
    assert a.reason == b.reason == 2 and a.its == b.its and a.outer_its == b.outer_its
    # the outer FP64 residual after a refinement step is what the FP32 inner
    # solve reached, which the other summation order of p.w perturbs at the
    # level of FP32 rounding (a few per cent of the last residual, measured):
    # both start alike and both meet rtol
    ha, hb = a.history(), b.history()
    assert len(ha) == len(hb) and ha[0] == hb[0]
    rtol = 1e-12 if "1e-12" in args else 1e-10
    assert a.true_rel_resid <= rtol and b.true_rel_resid <= rtol
    d = (u1 - u0).abs().max().item()
    assert d <= 1e-9 * u0.abs().max().item()
    assert abs(a.errinf - b.errinf) <= 1e-9 * u0.abs().max().item()


@pytest.mark.parametrize("args", [
    "-fsh_dim 2 -fsh_problem manupoly -da_refine 7 -pc_type mg -mg_levels_ksp_type chebyshev "
    "-mg_levels_pc_type jacobi -ksp_rtol 1e-10",
    "-fsh_dim 2 -fsh_problem manupoly -da_refine 8 -pc_type mg -ksp_rtol 1e-10 -fsh_precision mixed",
    "-fsh_dim 2 -fsh_problem manupoly -da_grid_x 5 -da_grid_y 3 -da_refine 7 -pc_type mg -ksp_rtol 1e-10 -fsh_cy 3",
    "-fsh_dim 3 -fsh_problem manupoly -da_refine 5 -pc_type mg -ksp_rtol 1e-10",
    "-fsh_dim 3 -fsh_problem manuexp -da_refine 6 -pc_type mg -ksp_rtol 1e-10 -fsh_precision mixed",
    "-fsh_dim 3 -fsh_problem manupoly -da_grid_x 3 -da_grid_y 5 -da_grid_z 9 -da_refine 3 -pc_type mg "
    "-ksp_rtol 1e-10 -fsh_cz 2 -ksp_norm_type unpreconditioned",
    "-fsh_dim 3 -fsh_problem manupoly -da_grid_x 3 -da_grid_y 5 -da_grid_z 9 -da_refine 3 -pc_type mg "
    "-ksp_rtol 1e-10 -fsh_cz 2 -fsh_precision mixed",
])
def test_vcycle_tail_is_bit_identical(cuda, args):
    """The V-cycle's small levels in one block (k_vtail) compute every point
    with the operations of the per-phase kernels, in the same order: the
    solve is identical, bit for bit, to the launch-per-phase form."""
    import torch
    fg = fgmod()
    u1, a = fg.solve(fg.options(args + " -fsh_vtail 1 -fsh_persist 0"))
    u0, b = fg.solve(fg.options(args + " -fsh_vtail 0 -fsh_persist 0"))
    assert a.reason == b.reason == 2 and a.its == b.its and a.outer_its == b.outer_its
    assert a.history() == b.history()
    assert torch.equal(u1, u0)
    assert a.launches <= b.launches  # fewer wherever a level is small enough for the tail


@pytest.mark.parametrize("args", [
    "-fsh_dim 2 -fsh_problem manupoly -da_refine 8 -pc_type mg -mg_levels_ksp_type chebyshev "
    "-mg_levels_pc_type jacobi -ksp_rtol 1e-10 -fsh_coop_tail -1",
    "-fsh_dim 2 -fsh_problem manupoly -da_refine 9 -pc_type mg -ksp_rtol 1e-10 -fsh_precision mixed -fsh_coop_tail -1",
    "-fsh_dim 2 -fsh_problem manupoly -da_grid_x 5 -da_grid_y 3 -da_refine 7 -pc_type mg -ksp_rtol 1e-10 -fsh_cy 3 "
    "-ksp_norm_type unpreconditioned -fsh_coop_tail 20000",
    "-fsh_dim 3 -fsh_problem manupoly -da_refine 6 -pc_type mg -ksp_rtol 1e-10 -fsh_coop_tail -1",
    "-fsh_dim 3 -fsh_problem manuexp -da_refine 6 -pc_type mg -ksp_rtol 1e-10 -fsh_precision mixed -fsh_coop_tail -1",
    "-fsh_dim 3 -fsh_problem manupoly -da_grid_x 3 -da_grid_y 5 -da_grid_z 9 -da_refine 3 -pc_type mg "
    "-ksp_rtol 1e-10 -fsh_cz 2 -fsh_precision mixed -fsh_coop_tail 6000",
])
def test_cooperative_vcycle_tail_is_bit_identical(cuda, args):
    """The V-cycle's levels from the largest of at most coop_tail nodes down as
    one cooperative launch (k_vtail_coop, persist_vcycle's phases with a
    grid-wide barrier between them; an option, off by default) compute every
    point with the operations of the per-phase kernels: the launch-per-phase
    solve is identical, bit for bit, with and without it, in fewer launches."""
    import torch
    fg = fgmod()
    u1, a = fg.solve(fg.options(args + " -fsh_persist 0"))
    u0, b = fg.solve(fg.options(args + " -fsh_persist 0 -fsh_coop_tail 0"))
    assert a.reason == b.reason == 2 and a.its == b.its and a.outer_its == b.outer_its
    assert a.history() == b.history()
    assert torch.equal(u1, u0)
    assert a.launches < b.launches


@pytest.mark.parametrize("args", [
    "-fsh_dim 3 -fsh_problem manupoly -da_refine 6 -pc_type mg -ksp_rtol 1e-10 -fsh_precision mixed",
    "-fsh_dim 3 -fsh_problem manuexp -da_grid_x 5 -da_grid_y 3 -da_grid_z 9 -da_refine 4 -pc_type mg "
    "-ksp_rtol 1e-10 -fsh_precision mixed -fsh_inner_accurate 1",
    "-fsh_dim 2 -fsh_problem manupoly -da_refine 9 -pc_type mg -ksp_rtol 1e-10 -fsh_precision mixed",
    "-fsh_dim 2 -fsh_problem manupoly -da_refine 8 -pc_type mg -ksp_rtol 1e-10 -fsh_precision mixed "
    "-fsh_inner_accurate 1 -fsh_graph_iters 4 -fsh_device_loop 0",
])
def test_paired_y_updates_are_bit_identical(cuda, args):
    """The accurate inner form updates its FP64 correction every other CG
    iteration, two steps at a time, fma(a, p_old, fma(a2, p_older, y)): the
    values of one update per iteration (the FP64 intermediate is what y would
    have held), so the solve is identical, bit for bit, to -fsh_pair_y 0 --
    whatever iteration the inner solves stop at (an update may still be owed
    from two iterations back)."""
    import torch
    fg = fgmod()
    u1, a = fg.solve(fg.options(args + " -fsh_persist 0"))
    u0, b = fg.solve(fg.options(args + " -fsh_persist 0 -fsh_pair_y 0"))
    assert a.reason == b.reason == 2 and a.its == b.its and a.outer_its == b.outer_its
    assert a.history() == b.history()
    assert torch.equal(u1, u0)


PERSIST_CASES = [
    # fish's 2D case (preconditioned norm), FP64 and mixed
    "-fsh_dim 2 -fsh_problem manupoly -da_refine 7 -pc_type mg -mg_levels_ksp_type chebyshev "
    "-mg_levels_pc_type jacobi -ksp_rtol 1e-10",
    "-fsh_dim 2 -fsh_problem manupoly -da_refine 7 -pc_type mg -ksp_rtol 1e-10 -fsh_precision mixed",
    # uneven anisotropic 2D grid, unpreconditioned norm
    "-fsh_dim 2 -fsh_problem manupoly -da_grid_x 5 -da_grid_y 3 -da_refine 6 -pc_type mg -ksp_rtol 1e-10 -fsh_cy 3 "
    "-ksp_norm_type unpreconditioned",
    # 3D, both forms, the accurate inner form forced on and off
    "-fsh_dim 3 -fsh_problem manupoly -da_refine 5 -pc_type mg -ksp_rtol 1e-10",
    "-fsh_dim 3 -fsh_problem manuexp -da_grid_x 5 -da_grid_y 3 -da_grid_z 9 -da_refine 3 -pc_type mg -ksp_rtol 1e-10 "
    "-fsh_precision mixed -fsh_inner_accurate 1",
    "-fsh_dim 3 -fsh_problem manupoly -da_refine 5 -pc_type mg -ksp_rtol 1e-10 -fsh_precision mixed "
    "-fsh_inner_accurate 0",
    # the whole hierarchy but the coarsest level in the grid-wide part
    "-fsh_dim 2 -fsh_problem manupoly -da_refine 6 -pc_type mg -ksp_rtol 1e-10 -fsh_persist_tail 25",
    # random initial state (a nonzero initial iterate)
    "-fsh_dim 3 -fsh_problem manupoly -da_refine 4 -pc_type mg -fsh_initial_type random -fsh_seed 77 -ksp_rtol 1e-10",
]


@pytest.mark.parametrize("args", PERSIST_CASES)
def test_persistent_solve_matches_the_launch_per_phase_solve(cuda, args):
    """The whole CG + MG solve as one cooperative launch (k_ksp_persist) runs
    every point with the per-phase kernels' operations; only the dot
    products are summed in another order.  FP64: the same iterations and the
    history to 1e-10 relative; mixed: the same refinement steps, both meet
    rtol, solutions to 1e-9 relative of max|u|."""
    fg = fgmod()
    u1, a = fg.solve(fg.options(args + " -fsh_persist 1"))
    u0, b = fg.solve(fg.options(args + " -fsh_persist 0"))
    assert a.reason == b.reason == 2 and a.outer_its == b.outer_its
    assert a.launches < b.launches  # the persistent path was taken
    scale = u0.abs().max().item()
    if "mixed" in args:
        assert abs(a.its - b.its) <= 1
        assert a.true_rel_resid <= 1e-10 and b.true_rel_resid <= 1e-10
        assert a.history()[0] == b.history()[0]
        d = (u1 - u0).abs().max().item()
        assert d <= 1e-9 * scale, d
    else:
        assert a.its == b.its
        ha, hb = a.history(), b.history()
        assert len(ha) == len(hb)
        for x, y in zip(ha, hb):
            assert abs(x - y) <= 1e-10 * abs(y) + 1e-14 * hb[0]
        d = (u1 - u0).abs().max().item()
        assert d <= 1e-10 * scale, d
    assert abs(a.errinf - b.errinf) <= 1e-8 * scale


@pytest.mark.parametrize("args", [PERSIST_CASES[0], PERSIST_CASES[2], PERSIST_CASES[3]])
def test_persistent_solve_matches_oracle(cuda, args):
    """The persistent FP64 solve against the CPU oracle, as the launch-per-phase
    solves are compared (compare_runs: iterations, reason, history to 1e-8,
    errors), and the solution within 1e-9 of max|u|."""
    fg = fgmod()
    u, rep = fg.solve(fg.options(args + " -fsh_persist 1"))
    uref, ref = orc.fish_solve(orc.options(args.split()))
    compare_runs(args.split(), rep, ref)
    diff = np.max(np.abs(u.cpu().numpy() - uref))
    assert diff <= 1e-9 * max(1e-300, np.max(np.abs(uref)))


def test_persistent_solve_is_deterministic_and_reusable(cuda):
    import torch
    fg = fgmod()
    o = fg.options(PERSIST_CASES[1] + " -fsh_persist 1")
    with fg.Solver(o) as s:
        u1 = torch.empty(o.shape, dtype=torch.float64, device=cuda)
        u2 = torch.empty_like(u1)
        r1 = s.solve(u1)
        r2 = s.solve(u2)
    assert r1.its == r2.its and r2.launches < 12  # one launch per inner solve, a few around them
    assert torch.equal(u1, u2) and r1.history() == r2.history()


@pytest.mark.parametrize("args", [
    "-fsh_dim 3 -fsh_problem manupoly -da_refine 5 -pc_type mg -ksp_rtol 1e-10 -fsh_precision mixed",
    "-fsh_dim 3 -fsh_problem manuexp -da_refine 4 -pc_type mg -ksp_rtol 1e-10 -fsh_precision mixed "
    "-fsh_inner_accurate 0",
    "-fsh_dim 2 -fsh_problem manupoly -da_grid_x 5 -da_grid_y 3 -da_refine 6 -pc_type mg -ksp_rtol 1e-10 "
    "-fsh_cy 3 -fsh_precision mixed",
    "-fsh_dim 3 -fsh_problem manupoly -da_grid_x 3 -da_grid_y 5 -da_grid_z 9 -da_refine 3 -pc_type mg "
    "-pc_mg_cycle_type w -ksp_rtol 1e-10 -fsh_precision mixed -fsh_inner_accurate 1",
    "-fsh_dim 1 -fsh_problem manupoly -da_refine 8 -pc_type mg -ksp_rtol 1e-10 -fsh_precision mixed",
])
def test_fused_residual_update_is_bit_identical(cuda, args):
    """r -= alpha w carried into the V-cycle's first smoothing pass (the
    residual formed on the fly as v_cg_r forms it, r.r reduced over the same
    slots in the same order): the solve is identical, bit for bit, to the
    separate update, with one launch fewer per iteration."""
    import torch
    fg = fgmod()
    u1, a = fg.solve(fg.options(args + " -fsh_fuse_cgr 1 -fsh_persist 0"))
    u0, b = fg.solve(fg.options(args + " -fsh_fuse_cgr 0 -fsh_persist 0"))
    assert a.reason == b.reason == 2 and a.its == b.its and a.outer_its == b.outer_its
    assert a.history() == b.history()
    assert torch.equal(u1, u0)
    assert a.launches < b.launches


def test_persistent_solves_on_concurrent_streams(cuda):
    """Two persistent solves launched on two streams at once (cooperative
    launches that each want every SM): both complete with the results of the
    same solves run alone."""
    import threading
    import torch
    fg = fgmod()
    args = [PERSIST_CASES[0] + " -fsh_persist 1", PERSIST_CASES[3] + " -fsh_persist 1"]
    alone = [fg.solve(fg.options(a)) for a in args]
    streams = [torch.cuda.Stream(device=cuda) for _ in args]
    opts = [fg.options(a) for a in args]
    solvers = [fg.Solver(o, stream=st.cuda_stream) for o, st in zip(opts, streams)]
    us = [torch.empty(o.shape, dtype=torch.float64, device=cuda) for o in opts]
    reps = [None, None]

    def run(q):
        for _ in range(3):
            reps[q] = solvers[q].solve(us[q])

    th = [threading.Thread(target=run, args=(q,)) for q in range(2)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    torch.cuda.synchronize()
    for q in range(2):
        ua, ra = alone[q]
        assert reps[q].reason == ra.reason == 2 and reps[q].its == ra.its
        assert torch.equal(us[q], ua)
        solvers[q].close()


@pytest.mark.parametrize("args", [
    # the iteration cap stops the FP64 CG (DIVERGED_ITS), mid-V-cycle state left behind
    "-fsh_dim 2 -fsh_problem manupoly -da_refine 6 -pc_type mg -ksp_rtol 1e-12 -ksp_max_it 3",
    # the mixed form's outer cap and inner cap
    "-fsh_dim 3 -fsh_problem manupoly -da_refine 4 -pc_type mg -ksp_rtol 1e-12 -fsh_precision mixed "
    "-fsh_outer_max_it 1",
    "-fsh_dim 2 -fsh_problem manupoly -da_refine 6 -pc_type mg -ksp_rtol 1e-12 -fsh_precision mixed "
    "-fsh_inner_max_it 2",
    # a zero right-hand side: converged before any iteration
    "-fsh_dim 3 -fsh_problem zero -da_refine 4 -pc_type mg -ksp_rtol 1e-10 -fsh_precision mixed",
])
def test_persistent_solve_stops_as_the_launch_per_phase_solve(cuda, args):
    """The persistent solves stop for the same reasons as the launch-per-phase
    solves (caps, a zero right-hand side), with the same reports: FP64 the
    same iterations and history to 1e-10; mixed the same refinement steps,
    inner iterations within one per step (an FP32 dot product summed in
    another order can move a stop by one iteration), history to 1e-3."""
    fg = fgmod()
    u1, a = fg.solve(fg.options(args + " -fsh_persist 1"))
    u0, b = fg.solve(fg.options(args + " -fsh_persist 0"))
    mixed = "mixed" in args
    assert a.reason == b.reason and a.outer_its == b.outer_its, (a.reason, b.reason, a.outer_its, b.outer_its)
    assert abs(a.its - b.its) <= (max(1, b.outer_its) if mixed else 0), (a.its, b.its)
    assert a.launches < b.launches or b.launches <= 6
    ha, hb = a.history(), b.history()
    assert len(ha) == len(hb)
    tol = 1e-3 if mixed else 1e-10
    for x, y in zip(ha, hb):
        assert abs(x - y) <= tol * abs(y) + 1e-14 * max(hb[0], 1e-300), (x, y)
    scale = max(u0.abs().max().item(), 1e-300)
    assert (u1 - u0).abs().max().item() <= (1e-3 if mixed else 1e-10) * scale
