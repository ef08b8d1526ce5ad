"""CPU tests of the serving-stream generator: sizes are multigrid sizes in
the stated ranges, rounding is nearest in log2(n - 1), arrivals are a
Poisson process at the requested rate, and the stream is reproducible."""
import numpy as np

from p4pdes_gb300 import serve


def test_round_size():
    assert [serve.round_size(n) for n in (65, 90, 97, 100, 129, 1025, 33, 40, 50)] == \
        [65, 65, 129, 129, 129, 1025, 33, 33, 65]


def test_stream_sizes_rate_and_reproducibility():
    s = serve.make_stream(4000, rate=2000.0, seed=2)
    assert s == serve.make_stream(4000, rate=2000.0, seed=2)
    t = np.array([a for a, _, _ in s])
    assert t[0] == 0.0 and np.all(np.diff(t) >= 0)
    assert abs(len(s) / t[-1] - 2000.0) < 100.0
    for _, d, n in s:
        lo, hi = serve.DIMS_RANGE[d]
        assert lo <= n <= hi and ((n - 1) & (n - 2)) == 0
    dims = [d for _, d, _ in s]
    assert 0.45 < dims.count(2) / len(dims) < 0.55
    # end sizes get about half the weight of inner ones
    n2 = [n for _, d, n in s if d == 2]
    assert 0.3 < n2.count(65) / n2.count(257) < 0.7


def test_output_arena_gives_disjoint_aligned_arrays():
    s = serve.make_stream(40, seed=5)
    b = serve._Buffers(s, 2, 3, pinned=False)
    base = b.arena.ctypes.data
    spans = []
    for (_, d, n), u in zip(s, b.outs):
        assert u.shape == (n,) * d and u.flags["C_CONTIGUOUS"]
        off = u.ctypes.data - base
        assert off % 512 == 0
        spans.append((off, off + 8 * n ** d))
    spans.sort()
    assert all(a[1] <= b_[0] for a, b_ in zip(spans, spans[1:]))
    assert all(len(v) == 2 for v in b.rhs.values())
