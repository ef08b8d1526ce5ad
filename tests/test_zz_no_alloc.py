"""PoissonOperatorApplyNoAlloc_gpu: the allocation-free form of the Jacobian
apply + dot, for callers that may not allocate device memory once running.

It is called through the C ABI twice in a row (the static scratch keeps the
previous call's contents, so the second call checks that nothing stale leaks
into the dot product) and compared with Poisson{1,2,3}DOperatorApply_gpu to
the tolerance the other apply tests use: 1e-13 relative for q, 1e-12 for p.q.
The file sorts last so a run that stops at the first failure has already run
every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dim,m", [(1, (257, 1, 1)), (2, (129, 65, 1)), (3, (65, 33, 129))])
def test_no_alloc_apply_matches_allocating_apply(cuda, dim, m):
    import torch
    import p4pdes_gb300 as fg
    lib = fg.load()
    inf = fg.Info()
    inf.dim, (inf.mx, inf.my, inf.mz) = dim, m
    inf.xm, inf.ym, inf.zm = m
    inf.xmax[0], inf.xmax[1], inf.xmax[2] = 1.0, 2.0, 0.5
    ctx = fg.Ctx()
    ctx.Lx, ctx.Ly, ctx.Lz, ctx.cx, ctx.cy, ctx.cz = 1.0, 2.0, 0.5, 1.0, 0.7, 3.0
    ctx.problem, ctx.dim = fg.ZERO, dim
    shape = (m[2], m[1], m[0])
    gen = torch.Generator(device="cpu").manual_seed(dim)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        p = torch.randn(shape, dtype=torch.float64, generator=gen).cuda()
        q_ref = torch.empty_like(p)
        d_ref = torch.zeros(1, dtype=torch.float64, device=cuda)
        rc = getattr(lib, "Poisson%dDOperatorApply_gpu" % dim)(ctypes.byref(inf), p.data_ptr(), q_ref.data_ptr(),
                                                              d_ref.data_ptr(), ctypes.byref(ctx), stream)
        assert rc == 0
        q = torch.full_like(p, float("nan"))
        d = torch.full((1,), float("nan"), dtype=torch.float64, device=cuda)
        rc = lib.PoissonOperatorApplyNoAlloc_gpu(ctypes.byref(inf), p.data_ptr(), q.data_ptr(), d.data_ptr(),
                                                 ctypes.byref(ctx), stream)
        assert rc == 0, "call %d" % call
        torch.cuda.synchronize()
        qr, qn = q_ref.cpu().numpy(), q.cpu().numpy()
        assert np.max(np.abs(qn - qr)) <= 1e-13 * np.max(np.abs(qr)), "call %d" % call
        dr = d_ref.item()
        assert abs(d.item() - dr) <= 1e-12 * abs(dr), (call, d.item(), dr)
