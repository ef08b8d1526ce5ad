"""GPU tests of the solve server (continuous batching of independent solves
of uneven sizes, 2D and 3D): each result is bit-identical to the same request
solved alone on a fresh solver (tolerance 0: per-request state, deterministic
reductions, nothing shared between concurrent solves), every request meets
rtol on its FP64 true residual recomputed on the CPU, a small HBM budget still
completes every request by evicting idle solvers, and the device-memory
estimate used for admission equals what a solver allocates."""
import numpy as np
import pytest

import _oracle as orc

pytestmark = pytest.mark.gpu


def requests(seed=2):
    rng = np.random.default_rng(seed)
    sizes = [(2, 33), (3, 17), (2, 129), (3, 33), (2, 65), (2, 257), (3, 65), (2, 33), (3, 17), (2, 129),
             (3, 33), (2, 65), (2, 9), (3, 9)]
    return [(d, n, rng.standard_normal((n,) * d)) for d, n in sizes]


def solve_alone(dim, n, f, rtol=1e-8):
    import p4pdes_gb300 as fg
    u = np.full_like(f, np.nan)
    with fg.Solver(fg.server_request_opts(dim, n, rtol)) as s:
        rep = s.solve_host(f, None, u)
    return u, rep


def relres_cpu(dim, n, f, u):
    """||b - A u|| / ||b|| in FP64 with the oracle's operator, b = h^dim f
    inside and 0 on the boundary (fish.c's scaling of the right-hand side)."""
    g = orc.grid(dim, n, n if dim >= 2 else 1, n if dim >= 3 else 1, problem=orc.ZERO)
    h = 1.0 / (n - 1)
    b = (h ** dim) * f.copy()
    for ax in range(dim):
        sl = [slice(None)] * dim
        sl[ax] = 0
        b[tuple(sl)] = 0.0
        sl[ax] = -1
        b[tuple(sl)] = 0.0
    shp = orc.shape(g)
    r = b.reshape(shp) - orc.apply(g, np.ascontiguousarray(u.reshape(shp)))
    return np.linalg.norm(r) / np.linalg.norm(b)


def run_server(reqs, **kw):
    import p4pdes_gb300 as fg
    us = [np.full_like(f, np.nan) for _, _, f in reqs]
    with fg.Server(**kw) as srv:
        tickets = [srv.submit(d, n, f, u) for (d, n, f), u in zip(reqs, us)]
        res = [srv.wait(t, 120000.0) for t in tickets]
        stats = srv.stats()
    return us, res, stats


def test_mixed_stream_equals_each_request_alone(cuda):
    """Every request its own solver (batch_max 1): bit-identical to a fresh
    solver."""
    reqs = requests()
    us, res, stats = run_server(reqs, workers=6, batch_max=1)
    assert stats["created"] >= len({(d, n) for d, n, _ in reqs})
    for (d, n, f), u, r in zip(reqs, us, res):
        assert r.status == 0 and r.rel_resid <= 1e-8, (d, n, r.status, r.rel_resid)
        assert r.latency_ms >= r.service_ms > 0.0 and r.queue_ms >= 0.0
        ua, rep = solve_alone(d, n, f)
        assert np.array_equal(u, ua), (d, n, np.max(np.abs(u - ua)))
        assert rep.its == r.its and rep.outer_its == r.outer_its
        assert relres_cpu(d, n, f, u) <= 2e-8


def test_small_budget_evicts_and_still_completes(cuda):
    import p4pdes_gb300 as fg
    reqs = requests(5)[:8]
    need = max(fg.estimate_bytes(fg.server_request_opts(d, n)) for d, n, _ in reqs)
    us, res, stats = run_server(reqs, workers=4, hbm_budget_bytes=need + need // 4, batch_max=1)
    assert stats["evicted"] > 0 and stats["pooled_bytes"] <= need + need // 4
    for (d, n, f), u, r in zip(reqs, us, res):
        assert r.status == 0
        ua, _ = solve_alone(d, n, f)
        assert np.array_equal(u, ua), (d, n)


def test_request_larger_than_budget_is_refused(cuda):
    import p4pdes_gb300 as fg
    f = np.zeros((257, 257))
    u = np.zeros_like(f)
    assert fg.estimate_bytes(fg.server_request_opts(2, 257)) > 1 << 20
    with fg.Server(hbm_budget_bytes=1 << 20, workers=1) as srv:
        with pytest.raises(fg.FishError) as e:
            srv.submit(2, 257, f, u)
        assert e.value.code == 3
        with pytest.raises(fg.FishError):
            srv.submit(2, 64, f, u)  # not 2^k + 1


@pytest.mark.parametrize("dim,n,prec", [(2, 129, 1), (3, 33, 1), (3, 33, 0), (2, 1025, 1), (3, 129, 1)])
def test_estimate_equals_allocation(cuda, dim, n, prec):
    import p4pdes_gb300 as fg
    o = fg.server_request_opts(dim, n, precision=prec)
    est = fg.estimate_bytes(o)
    f = np.random.default_rng(0).standard_normal((n,) * dim)
    u = np.empty_like(f)
    with fg.Solver(o) as s:
        s.solve_host(f, None, u)
        assert s.device_bytes == est


def test_same_size_2d_requests_are_merged_into_group_solves(cuda):
    """2D requests of one size queued together run as one group solve (the
    batch's plane-stacked kernels); each result is bit-identical to the same
    request solved alone in a group of one, meets rtol on the FP64 residual
    recomputed on the CPU, and 3D requests keep their own solvers."""
    import p4pdes_gb300 as fg
    rng = np.random.default_rng(11)
    sizes = [(2, 65)] * 6 + [(2, 129)] * 5 + [(3, 17)] * 2 + [(2, 33)] * 3
    reqs = [(d, n, rng.standard_normal((n,) * d)) for d, n in sizes]
    # one worker: everything queues behind the first request and is merged
    us, res, stats = run_server(reqs, workers=1, batch_max=4)
    assert stats["group_solves"] >= 1 and stats["grouped_requests"] > stats["group_solves"]
    assert stats["grouped_requests"] == sum(1 for d, _, _ in reqs if d == 2)
    for (d, n, f), u, r in zip(reqs, us, res):
        assert r.status == 0 and r.rel_resid <= 1e-8, (d, n, r.status, r.rel_resid)
        assert relres_cpu(d, n, f, u) <= 2e-8
        if d == 2:
            ua = np.full_like(f, np.nan)
            with fg.Group(n, 1) as g:
                (its, outer, rel), = g.solve_host([f], [ua])
            assert np.array_equal(u, ua), (n, np.max(np.abs(u - ua)))
            assert its == r.its and outer == r.outer_its
        else:
            ua, rep = solve_alone(d, n, f)
            assert np.array_equal(u, ua)


def test_group_instances_do_not_depend_on_the_group(cuda):
    """One instance in groups of 1, 3 (padded to 4) and 8: identical results."""
    import p4pdes_gb300 as fg
    rng = np.random.default_rng(3)
    fs = [rng.standard_normal((129, 129)) for _ in range(8)]
    outs = {}
    for count, k in ((1, 1), (4, 3), (8, 8)):
        us = [np.full_like(f, np.nan) for f in fs[:k]]
        with fg.Group(129, count) as g:
            r = g.solve_host(fs[:k], us)
        outs[count] = (us[0], r[0])
    for count in (4, 8):
        assert np.array_equal(outs[count][0], outs[1][0])
        assert outs[count][1] == outs[1][1]
    assert outs[1][1][2] <= 1e-8
