"""GPU tests of the batch solver (many independent 2D problems of uneven
sizes, -Laplace(u) = f, u = 0 on the boundary): every instance converges to
rtol on its FP64 true residual, matches the exact discrete solution computed
by the CPU oracle, and gives bit-identical results alone and in a mixed batch
(per-instance state, reductions and scales; nothing is shared between
instances)."""
import numpy as np
import pytest

import _oracle as orc

pytestmark = pytest.mark.gpu


def make_f(sizes, seed):
    rng = np.random.default_rng(seed)
    return [rng.standard_normal((n, n)) for n in sizes]


def solve_batch(fs, rtol=1e-8, tune=True):
    import torch
    import p4pdes_gb300 as fg
    sizes = [f.shape[0] for f in fs]
    ft = [torch.from_numpy(f).cuda() for f in fs]
    ut = [torch.full_like(f, float("nan")) for f in ft]
    with fg.Batch(sizes, rtol=rtol, tune=tune) as b:
        rep = b.solve(ft, ut)
        res = b.results()
    torch.cuda.synchronize()
    return [u.cpu().numpy() for u in ut], rep, res


def oracle_check(f, u, rtol):
    n = f.shape[0]
    g = orc.grid(2, n, n, problem=orc.ZERO)
    h = 1.0 / (n - 1)
    b = h * h * f
    b[0, :] = b[-1, :] = b[:, 0] = b[:, -1] = 0.0
    b = np.ascontiguousarray(b[None])
    r = b - orc.apply(g, np.ascontiguousarray(u[None]))
    rel = np.linalg.norm(r) / np.linalg.norm(b)
    ustar = orc.exact_solve(g, b)[0]
    return rel, np.max(np.abs(u - ustar)) / np.max(np.abs(ustar))


def test_batch_of_uneven_sizes_converges_and_matches_exact(cuda):
    sizes = [33, 9, 65, 17, 33, 5, 129, 9, 17, 65, 33, 3]
    fs = make_f(sizes, 1)
    us, rep, (inner, outer, rel, reason) = solve_batch(fs)
    assert rep.ninst == len(sizes) and rep.converged == len(sizes) and rep.groups == len(set(sizes))
    for q, (f, u) in enumerate(zip(fs, us)):
        assert reason[q] in (2, 3) and rel[q] <= 1e-8  # 3x3 is solved exactly (atol)
        assert not np.isnan(u).any()
        relres, relerr = oracle_check(f, u, 1e-8)
        assert relres <= 2e-8, (q, relres)          # recomputed independently in FP64 on the CPU
        assert relerr <= 1e-5, (q, relerr)
        # boundary rows scdiag*u = 0 hold to the solve's residual level
        edge = np.concatenate([u[0, :], u[-1, :], u[:, 0], u[:, -1]])
        assert np.max(np.abs(edge)) <= 1e-8 * np.max(np.abs(u))


def test_instance_alone_and_in_the_mix_is_identical(cuda):
    fs = make_f([65, 33, 129, 65, 17], 7)
    mix, _, _ = solve_batch(fs, tune=False)
    alone, _, _ = solve_batch([fs[0]], tune=False)
    assert np.array_equal(mix[0], alone[0])
    alone2, _, _ = solve_batch([fs[2]], tune=False)
    assert np.array_equal(mix[2], alone2[0])


def test_batch_with_tuned_blocks_agrees(cuda):
    fs = make_f([129, 65, 33, 33], 3)
    a, _, _ = solve_batch(fs, tune=False)
    b, _, _ = solve_batch(fs, tune=True)
    for x, y in zip(a, b):
        assert np.max(np.abs(x - y)) <= 1e-6 * np.max(np.abs(x))


def test_batch_rejects_sizes_that_do_not_coarsen(built):
    import p4pdes_gb300 as fg
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a device")
    with pytest.raises(fg.FishError):
        fg.Batch([33, 34])


def test_autotuner_picks_sweeps_per_group_and_every_instance_converges(cuda):
    """With tuning on, the smoothing steps of every size group are chosen by
    timing batched solves (1, 2 or 3 per level); the tuned batch still meets
    rtol on every instance, checked by the oracle.  Without sweep tuning every
    group keeps the batch's own count."""
    import torch
    import p4pdes_gb300 as fg
    sizes = [65, 33, 129, 65, 17, 33]
    fs = make_f(sizes, 5)
    ft = [torch.from_numpy(f).cuda() for f in fs]
    ut = [torch.full_like(f, float("nan")) for f in ft]
    with fg.Batch(sizes, rtol=1e-8, tune=True) as b:
        groups = b.groups()
        rep = b.solve(ft, ut)
    assert sorted(n for n, _, _ in groups) == sorted(set(sizes))
    assert all(sw in (1, 2, 3) for _, _, sw in groups)
    assert sum(c for _, c, _ in groups) == len(sizes)
    assert rep.converged == len(sizes)
    for f, u in zip(fs, ut):
        relres, _ = oracle_check(f, u.cpu().numpy(), 1e-8)
        assert relres <= 2e-8
    with fg.Batch(sizes, rtol=1e-8, tune=True, tune_sweeps=0) as b:
        assert all(sw == 2 for _, _, sw in b.groups())
