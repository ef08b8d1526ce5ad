"""PoissonOperatorApplyNoAlloc_gpu: the allocation-free form of the Jacobian
apply + dot, for callers that may not allocate device memory once running.

It is called through the C ABI twice in a row (the static scratch keeps the
previous call's contents, so the second call checks that nothing stale leaks
into the dot product) and compared with Poisson{1,2,3}DOperatorApply_gpu.  Both
run the same kernel with the same launch shape and summing order, so q and p.q
must be equal to the bit.  The allocating apply takes its scratch from the
device's default memory pool (cudaMallocAsync); the pool's high-water mark,
reset to zero before a no-alloc call, must still be zero after it.
The file sorts last so a run that stops at the first failure has already run
every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

POOL_USED_MEM_HIGH = 0x8  # cudaMemPoolAttrUsedMemHigh


def _cudart():
    rt = ctypes.CDLL("libcudart.so.13")
    rt.cudaDeviceGetDefaultMemPool.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int]
    rt.cudaMemPoolSetAttribute.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    rt.cudaMemPoolGetAttribute.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    return rt


def _pool_high(rt, pool, reset=False):
    v = ctypes.c_uint64(0)
    if reset:
        assert rt.cudaMemPoolSetAttribute(pool, POOL_USED_MEM_HIGH, ctypes.byref(v)) == 0
    assert rt.cudaMemPoolGetAttribute(pool, POOL_USED_MEM_HIGH, ctypes.byref(v)) == 0
    return v.value


@pytest.mark.parametrize("dim,m", [(1, (257, 1, 1)), (2, (129, 65, 1)), (3, (65, 33, 129))])
def test_no_alloc_apply_matches_allocating_apply(cuda, dim, m):
    import torch
    import p4pdes_gb300 as fg
    lib = fg.load()
    rt = _cudart()
    pool = ctypes.c_void_p()
    assert rt.cudaDeviceGetDefaultMemPool(ctypes.byref(pool), cuda.index or 0) == 0
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
        q = torch.full_like(p, float("nan"))
        d = torch.full((1,), float("nan"), dtype=torch.float64, device=cuda)
        torch.cuda.synchronize()
        _pool_high(rt, pool, reset=True)
        rc = getattr(lib, "Poisson%dDOperatorApply_gpu" % dim)(ctypes.byref(inf), p.data_ptr(), q_ref.data_ptr(),
                                                              d_ref.data_ptr(), ctypes.byref(ctx), stream)
        assert rc == 0
        torch.cuda.synchronize()
        assert _pool_high(rt, pool) > 0, "the allocating apply did not draw on the default pool"
        _pool_high(rt, pool, reset=True)
        rc = lib.PoissonOperatorApplyNoAlloc_gpu(ctypes.byref(inf), p.data_ptr(), q.data_ptr(), d.data_ptr(),
                                                 ctypes.byref(ctx), stream)
        assert rc == 0, "call %d" % call
        torch.cuda.synchronize()
        assert _pool_high(rt, pool) == 0, "call %d allocated from the default pool" % call
        assert np.array_equal(q.cpu().numpy(), q_ref.cpu().numpy()), "call %d" % call
        assert d.item() == d_ref.item(), (call, d.item(), d_ref.item())
