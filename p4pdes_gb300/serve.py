"""Serving workload: a Poisson-process stream of 2D and 3D solves of uneven
sizes fed to ``p4pdes_gb300.Server`` at their arrival times, with latency
percentiles and throughput.

Stream definition (mixed 2D/3D serving stream):
  * arrivals: exponential inter-arrival times with mean 1/rate, from
    ``numpy.random.default_rng(seed)`` (seed 2 by default);
  * dimension: 2 or 3 with probability 1/2 each (same generator);
  * size: n drawn log-uniform on [65, 1025] (2D) or [33, 257] (3D) and
    rounded to the nearest size the multigrid hierarchy needs, n = 2^k + 1
    with k = round(log2(n - 1)) (so the end sizes get half the weight of the
    inner ones);
  * right-hand side: iid N(0, 1) per node; each size has ``distinct_rhs``
    fields drawn from ``default_rng(seed + 1)`` and a request takes one of them
    at random (the server copies f to the device per request, so this bounds
    host memory without changing the work); every request has its own output
    array;
  * zero Dirichlet data, rtol 1e-8 on the FP64 true residual, mixed form.
"""
import math
import threading
import time

import numpy as np

DIMS_RANGE = {2: (65, 1025), 3: (33, 257)}


def round_size(n):
    """Nearest (in log2(n - 1)) size 2^k + 1."""
    return (1 << int(round(math.log2(n - 1)))) + 1


def make_stream(count, rate=2000.0, seed=2):
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=count))
    t -= t[0]
    out = []
    for q in range(count):
        dim = int(rng.integers(2, 4))
        lo, hi = DIMS_RANGE[dim]
        n = round_size(math.exp(rng.uniform(math.log(lo), math.log(hi))))
        out.append((float(t[q]), dim, n))
    return out


class _Buffers:
    """Host arrays: a few distinct right-hand sides per size, and one output
    array per request carved out of a single arena allocated before the
    stream starts (pinned when torch is available), so that no allocation
    happens while requests arrive."""

    def __init__(self, stream, distinct_rhs, seed, pinned):
        self.pinned = pinned
        rng = np.random.default_rng(seed)
        self.rhs = {}
        for key in sorted({(d, n) for _, d, n in stream}):
            d, n = key
            self.rhs[key] = [self._alloc(n ** d).reshape((n,) * d) for _ in range(distinct_rhs)]
            for a in self.rhs[key]:
                a[...] = self._from_numpy(rng.standard_normal((n,) * d))
        align = 64  # elements: 512-byte aligned views
        sizes = [-(-(n ** d) // align) * align for _, d, n in stream]
        self.arena = self._alloc(max(1, sum(sizes)))
        self.outs = []
        off = 0
        for (_, d, n), sz in zip(stream, sizes):
            self.outs.append(self.arena[off:off + n ** d].reshape((n,) * d))
            off += sz

    def _alloc(self, count):
        if self.pinned:
            import torch
            return torch.empty(count, dtype=torch.float64, pin_memory=True)
        return np.empty(count)

    def _from_numpy(self, a):
        if self.pinned:
            import torch
            return torch.from_numpy(a)
        return a


def run_stream(server, stream, distinct_rhs=4, seed=3, pinned=True):
    """Submits each request at its arrival time, waits for all, returns a
    summary: latency percentiles (arrival -> result on the host), solves/s and
    DOF/s over the whole stream (first arrival -> last completion)."""
    bufs = _Buffers(stream, distinct_rhs, seed, pinned)
    pick = np.random.default_rng(seed + 1).integers(0, distinct_rhs, size=len(stream))
    tickets = [None] * len(stream)
    results = [None] * len(stream)
    lag = [0.0] * len(stream)
    ready = threading.Semaphore(0)

    def waiter():
        for q in range(len(stream)):
            ready.acquire()
            results[q] = (server.wait(tickets[q]), time.perf_counter())

    th = threading.Thread(target=waiter, daemon=True)
    th.start()
    t0 = time.perf_counter()
    for q, (ta, d, n) in enumerate(stream):
        now = time.perf_counter() - t0
        if ta > now:
            time.sleep(ta - now)
        lag[q] = time.perf_counter() - t0 - ta
        tickets[q] = server.submit(d, n, bufs.rhs[(d, n)][pick[q]], bufs.outs[q])
        ready.release()
    th.join()
    t_end = max(r[1] for r in results)
    span = t_end - t0
    res = [r[0] for r in results]
    # latency from the request's arrival time: the submit thread's lag (when
    # it fell behind the arrival schedule) plus submit -> result
    lat = np.array([1e3 * lag[q] + r.latency_ms for q, r in enumerate(res)])
    lat_submit = np.array([r.latency_ms for r in res])
    svc = np.array([r.service_ms for r in res])
    dofs = sum(n ** d for _, d, n in stream)
    return {
        "requests": len(stream),
        "failed": int(sum(1 for r in res if r.status != 0)),
        "max_rel_resid": float(max(r.rel_resid for r in res)),
        "offered_rate": len(stream) / max(stream[-1][0], 1e-9),
        "span_s": span,
        "solves_per_s": len(stream) / span,
        "dofs_per_s": dofs / span,
        "p50_ms": float(np.percentile(lat, 50)),
        "p99_ms": float(np.percentile(lat, 99)),
        "mean_ms": float(lat.mean()),
        "submit_p50_ms": float(np.percentile(lat_submit, 50)),
        "submit_p99_ms": float(np.percentile(lat_submit, 99)),
        "service_p50_ms": float(np.percentile(svc, 50)),
        "service_p99_ms": float(np.percentile(svc, 99)),
        "max_submit_lag_ms": 1e3 * max(lag),
        "mean_outer_its": float(np.mean([r.outer_its for r in res])),
    }
