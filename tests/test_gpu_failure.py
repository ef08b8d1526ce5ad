"""Failure detection without a GPU fault.

The solvers' device-side loops (the CG and BiCGStab iterations as the body of
a conditional graph node) are capped: after `loop_cap` bodies the loop ends
whatever the solver's stop flag says, and the solve returns
FISHGPU_ERR_TIMEOUT instead of waiting for a flag that may never come.  Here
the cap is set below what the solve needs, so the cap runs out on purpose;
nothing spins, nothing faults, and the context stays usable (a solve right
after it on the same device gives the normal answer).  The server's wait
gives up with FISHGPU_ERR_TIMEOUT on a request that has not finished, and
the request still completes afterwards.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TIMEOUT = 6
FISH3D = ("-fsh_dim 3 -fsh_problem manupoly -da_refine 4 -pc_type mg -mg_levels_ksp_type chebyshev "
          "-mg_levels_pc_type jacobi -ksp_rtol 1e-10")


@pytest.mark.parametrize("extra", ["", "-fsh_precision mixed", "-fsh_device_loop 0",
                                   "-fsh_precision mixed -fsh_device_loop 0"])
def test_fish_loop_cap_ends_the_solve_with_timeout(cuda, extra):
    import torch
    import p4pdes_gb300 as fg
    # two CG iterations per loop body, so one body is less than any of these solves needs
    o = fg.options(FISH3D + " -fsh_graph_iters 2 -fsh_loop_cap 1 " + extra)
    u = torch.empty(o.shape, dtype=torch.float64, device=cuda)
    with fg.Solver(o) as s:
        with pytest.raises(fg.FishError) as e:
            s.solve(u)
        assert e.value.code == TIMEOUT
    # the device is still usable: the same solve without the cap converges
    o2 = fg.options(FISH3D + " " + extra)
    with fg.Solver(o2) as s:
        rep = s.solve(u)
    assert rep.reason == 2 and rep.its > 2


def test_fish_loop_cap_that_suffices_changes_nothing(cuda):
    """A cap above what the solve needs gives the same iterate, bit for bit."""
    import torch
    import p4pdes_gb300 as fg
    u1 = torch.empty(fg.options(FISH3D).shape, dtype=torch.float64, device=cuda)
    u2 = torch.empty_like(u1)
    with fg.Solver(fg.options(FISH3D)) as s:
        r1 = s.solve(u1)
    with fg.Solver(fg.options(FISH3D + " -fsh_loop_cap 50")) as s:
        r2 = s.solve(u2)
    assert r1.its == r2.its and r1.history() == r2.history()
    assert torch.equal(u1, u2)


def test_minimal_surface_loop_cap_ends_the_solve_with_timeout(cuda):
    import p4pdes_gb300 as fg
    with fg.MsSolver(fg.ms_options("-da_refine 3 -ksp_rtol 1e-10 -ms_loop_cap 1")) as s:
        with pytest.raises(fg.FishError) as e:
            s.solve()
        assert e.value.code == TIMEOUT
    with fg.MsSolver(fg.ms_options("-da_refine 3")) as s:
        rep = s.solve()
    assert rep.reason[0] > 0


def test_server_wait_gives_up_on_an_unfinished_request(cuda):
    import p4pdes_gb300 as fg
    rng = np.random.default_rng(7)
    f1, f2 = rng.standard_normal((129,) * 3), rng.standard_normal((129,) * 3)
    u1, u2 = np.full_like(f1, np.nan), np.full_like(f2, np.nan)
    # one worker: the second request waits in the queue behind the first
    with fg.Server(workers=1) as srv:
        t1 = srv.submit(3, 129, f1, u1)
        t2 = srv.submit(3, 129, f2, u2)
        with pytest.raises(fg.FishError) as e:
            srv.wait(t2, 0.0)
        assert e.value.code == TIMEOUT
        r1 = srv.wait(t1, -1.0)
        r2 = srv.wait(t2, -1.0)
    assert r1.status == 0 and r2.status == 0
    assert r2.rel_resid <= 1e-8 and np.all(np.isfinite(u2))


def test_persistent_grid_barrier_gives_up_and_the_device_stays_usable(cuda):
    """The persistent solve's grid barrier waits at most ~0.2 s: with one block
    absent (a flag nothing sets) the others give up, the fault word reports
    it, and the same solver then solves normally."""
    import time
    import torch
    import p4pdes_gb300 as fg
    o = fg.options("-fsh_dim 2 -fsh_problem manupoly -da_refine 7 -pc_type mg -ksp_rtol 1e-10 -fsh_persist 1")
    u = torch.empty(o.shape, dtype=torch.float64, device=cuda)
    with fg.Solver(o) as s:
        assert s.barrier_selftest(False) == 0
        t0 = time.perf_counter()
        assert s.barrier_selftest(True) == TIMEOUT
        assert time.perf_counter() - t0 < 5.0
        rep = s.solve(u)
        assert rep.reason == 2 and rep.launches < 12
