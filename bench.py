"""Benchmark: 3D Poisson 513^3 to 1e-10 relative residual, DOF/s.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (one step = one full fish solve): -fsh_dim 3 -fsh_problem manupoly
-da_refine 8 (513^3 nodes, 7-point), CG + MG V(2,2) Chebyshev/Jacobi on 9
levels, rtol 1e-10 on the true (unpreconditioned) residual.  `value` is the
mixed form (FP32 V-cycle and inner CG, FP64 iterative refinement) with f and g
resident in HBM; the plain FP64 form is measured beside it.  `e2e` is the same
K solves through fishgpu_solver_solve_host_many with pinned host arrays: every
step's f copied in, g read on the boundary and u copied out, the copies of
steps k+1 and k-1 overlapping the solve of step k; one fishgpu_solver_solve_host
call per step (copies serialised with the solve) is reported beside it.  Every
vector (1.08 GB in FP64) is far larger than L2, so no flush is needed between
steps.

--impl reference times the CPU restatement of the same solve (the oracle:
FP64 CG + MG, OpenMP on all host cores) on the same 513^3 workload, one whole
solve per step (about 6-7 s each on 16 Arm cores); its warm-up is one solve.
Multi-GPU: replicas only (independent solves per rank, no collective on the
data path); value = DOFs of all ranks / max time over ranks.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Poisson DOF/s to 1e-10 rel. residual, mixed vs FP64 MG, HBM %peak; p99 latency"
BASE_ARGS = ("-fsh_dim 3 -fsh_problem manupoly -da_refine {r} -pc_type mg -mg_levels_ksp_type chebyshev "
             "-mg_levels_pc_type jacobi -ksp_rtol 1e-10 -ksp_norm_type unpreconditioned")


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class Clocks:
    """nvidia-smi sampled every 200 ms during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        self.rows = []
        if self.p is None:
            return
        time.sleep(0.25)
        self.p.terminate()
        out, _ = self.p.communicate(timeout=10)
        for line in out.splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) == 6:
                self.rows.append(parts)

    def summary(self):
        if not getattr(self, "rows", None):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[q] for r in self.rows for q in range(4) if r[2 + q].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def cpu_baseline(refine, steps=None, budget_s=12.0):
    """Oracle (FP64 CG+MG, OpenMP on all host cores) on the bench's workload
    (-da_refine `refine`); `steps` whole solves, or as many as fit `budget_s`
    (at least one, at most five).  Returns (DOF/s, info)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import _oracle as orc
    o = orc.options(BASE_ARGS.format(r=refine).split())
    dofs = o.grid.mx * o.grid.my * o.grid.mz
    times = []
    t_all = time.perf_counter()
    n = 0
    while True:
        t0 = time.perf_counter()
        _, rep = orc.fish_solve(o)
        times.append(time.perf_counter() - t0)
        n += 1
        if steps is not None and n >= steps:
            break
        if steps is None and (time.perf_counter() - t_all > budget_s or n >= 5):
            break
    tot = sum(times)
    return dofs * n / tot, {"cores": orc.lib().or_num_threads(), "solves": n, "its": rep["its"], "dofs": dofs,
                            "errinf": rep["errinf"], "s_per_solve": tot / n,
                            "sample": "oracle FP64 CG+MG V(2,2) Chebyshev/Jacobi, 3D %d^3 manupoly, rtol 1e-10 "
                                      "(unpreconditioned norm), %d whole solve(s), %.2f s" % (o.grid.mx, n, tot)}


def job_rate(units_per_rank, ms_local, world, device):
    """Whole-job throughput of N replicas: every rank processed
    `units_per_rank`; the job took the slowest rank's time (max over ranks).
    Returns (units per second, max ms)."""
    import torch
    t = torch.tensor([float(ms_local)], dtype=torch.float64, device=device)
    if world > 1:
        import torch.distributed as dist
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms = t.item()
    return world * units_per_rank / (ms * 1e-3), ms


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


WORKLOAD = "3D Poisson 513^3 7-point (-da_refine 8), CG+MG V(2,2) Chebyshev/Jacobi, 9 levels, " \
           "rtol 1e-10 true residual"


def run_reference(args):
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    W = max(0, args.warmup)
    K = max(1, args.steps)
    for _ in range(min(W, 1)):  # one untimed solve warms the host (pages, threads)
        cpu_baseline(args.refine, steps=1)
    v, info = cpu_baseline(args.refine, steps=K)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "DOF/s", "n_gpus": args.gpus,
            "steps": K, "warmup": W, "ms_per_step": 1e3 * info["dofs"] / v,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (manufactured manupoly problem)",
            "config": {"workload": WORKLOAD, "dofs": info["dofs"], "levels": args.refine + 1,
                       "parallelism": "host cores (OpenMP)",
                       "measured_on": "the whole workload: one %d^3 solve per step, %d timed steps after %d "
                                      "untimed solve(s)" % (round(info["dofs"] ** (1 / 3)), K, min(W, 1)),
                       "its": info["its"], "errinf": info["errinf"],
                       "implementation": "CPU restatement (oracle) of the reference's CG + MG V(2,2) "
                                         "Chebyshev/Jacobi path, FP64; PETSc is not available to build "
                                         "the reference's own fish"},
            "cpu_baseline": {"value": v, "unit": "DOF/s", "cores": info["cores"], "kind": "port",
                             "sample": info["sample"]},
            "e2e": {"value": v, "unit": "DOF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def manupoly_fg(torch, o, dev):
    """f and g of the 3D manupoly problem (c/ch6/fish.c:23-25, :60-70) at every node."""
    mz, my, mx = o.shape
    x = torch.linspace(0, o.ctx.Lx, mx, dtype=torch.float64, device=dev).view(1, 1, mx)
    y = torch.linspace(0, o.ctx.Ly, my, dtype=torch.float64, device=dev).view(1, my, 1)
    z = torch.linspace(0, o.ctx.Lz, mz, dtype=torch.float64, device=dev).view(mz, 1, 1)
    aa, bb, cc = x * x * (1 - x * x), y * y * (y * y - 1), z * z * (z * z - 1)
    da, db, dc = 2 * (1 - 6 * x * x), 2 * (6 * y * y - 1), 2 * (6 * z * z - 1)
    g = (aa * bb * cc).contiguous()
    f = (-(da * bb * cc + aa * db * cc + aa * bb * dc)).contiguous()
    return f, g


def batch_leg(torch, fg, n_inst, reps=3):
    """4096 independent 2D instances, n = 2^k + 1 with k ~ U{5..9} from
    default_rng(0), f ~ N(0,1) per node from default_rng(1), u = 0 on the
    boundary, rtol 1e-8, mixed form; inputs resident on the device."""
    import numpy as np
    ks = np.random.default_rng(0).integers(5, 10, size=n_inst)
    sizes = [int(2 ** k + 1) for k in ks]
    frng = np.random.default_rng(1)
    fs = [torch.from_numpy(frng.standard_normal((n, n))).cuda() for n in sizes]
    us = [torch.empty_like(f) for f in fs]
    t0 = time.perf_counter()
    b = fg.Batch(sizes, rtol=1e-8, tune=True)
    b.solve(fs, us)  # warm-up (graphs, tuned chunk sizes)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    best = None
    for _ in range(reps):
        rep = b.solve(fs, us)
        if best is None or rep.solve_ms < best.solve_ms:
            best = rep
    inner, outer, rel, reason = b.results()
    groups = b.groups()
    b.close()
    return {
        "workload": "%d 2D Poisson instances, n = 2^k+1, k ~ U{5..9} (seed 0), f ~ N(0,1) (seed 1), rtol 1e-8, "
                    "mixed form, inputs resident" % n_inst,
        "solve_ms": best.solve_ms, "solves_per_s": n_inst / (best.solve_ms * 1e-3),
        "dofs": best.dofs, "dof_per_s": best.dofs / (best.solve_ms * 1e-3), "groups": best.groups,
        "converged": best.converged, "max_outer": best.max_outer, "max_inner": best.max_inner,
        "max_rel_resid": max(rel), "launches": best.launches, "setup_s": setup_s,
        "size_groups": [{"n": n, "instances": c, "smoothing_steps": sw} for n, c, sw in groups],
        "tuning": "tiles (block size, rows per thread) per level by timing a smoothing step; smoothing steps "
                  "per group by timing batched solves of up to 32 instances (part of setup_s)",
        "timing": "CUDA events around one batched solve, best of %d" % reps,
    }


def c1_leg(torch, fg, reps=20):
    """fish.c's own CPU-runnable case (2D manupoly 257^2, -da_refine 7, CG + 8-level MG V(2,2)
    Chebyshev/Jacobi, rtol 1e-10): the FP64 form (the reference's arithmetic) and the mixed form,
    iterations and discretisation error, beside the oracle's CPU time for the same FP64 solve."""
    args = ("-fsh_dim 2 -fsh_problem manupoly -da_refine 7 -pc_type mg -mg_levels_ksp_type chebyshev "
            "-mg_levels_pc_type jacobi -ksp_rtol 1e-10")
    out = {"workload": "2D Poisson, manupoly, 257^2 nodes, 8 MG levels, rtol 1e-10", "options": args}
    for prec in ("fp64", "mixed"):
        o = fg.options(args + " -fsh_precision " + prec)
        with fg.Solver(o) as s:
            u = torch.empty(o.shape, dtype=torch.float64, device="cuda")
            s.solve(u)
            ms = min(s.solve(u).solve_ms for _ in range(reps))
            rep = s.solve(u)
        out[prec] = {"ms": ms, "dof_per_s": o.dofs / (ms * 1e-3), "its": rep.its, "outer_its": rep.outer_its,
                     "errinf": rep.errinf, "err2h": rep.err2h}
    try:
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import _oracle as orc
        oo = orc.options(args.split())
        best = None
        for _ in range(3):
            t0 = time.perf_counter()
            _, r = orc.fish_solve(oo)
            dt = time.perf_counter() - t0
            best = dt if best is None or dt < best else best
        dofs = oo.grid.mx * oo.grid.my
        out["cpu_baseline"] = {"value": dofs / best, "unit": "DOF/s", "cores": orc.lib().or_num_threads(),
                               "kind": "port", "its": r["its"], "errinf": r["errinf"],
                               "sample": "oracle FP64 CG+MG on the same 257^2 solve, best of 3 (%.1f ms)" % (best * 1e3)}
    except Exception as e:  # oracle library missing: report why
        out["cpu_baseline"] = {"unavailable": str(e)[:200]}
    return out


def minimal_leg(fg, reps=3):
    """Minimal-surface equation (c/ch7/minimal.c), catenoid c = 1.1 on the unit
    square, 1025 x 1025 reached by grid sequencing from 33 x 33 (5 refinements),
    snes rtol 1e-10; the whole sequence is one solve."""
    import numpy as np
    args = "-da_grid_x 33 -da_grid_y 33 -snes_grid_sequence 5 -snes_rtol 1e-10"
    o = fg.ms_options(args)
    u = np.empty((1025, 1025))
    with fg.MsSolver(o) as s:
        s.solve(u)  # warm-up
        best = None
        for _ in range(reps):
            t0 = time.perf_counter()
            rep = s.solve(u)
            wall = time.perf_counter() - t0
            if best is None or rep.solve_ms < best[0].solve_ms:
                best = (rep, wall)
    rep, wall = best
    out = {
        "workload": "minimal surface, catenoid c=1.1 on the unit square, 33^2 -> 1025^2 by grid sequencing, "
                    "Newton + FP32 BiCGStab/Poisson-MG inner solves, FP64 residual, snes rtol 1e-10",
        "options": args, "dofs": rep.dofs, "solve_ms": rep.solve_ms, "wall_ms": wall * 1e3,
        "dof_per_s": rep.dofs / (rep.solve_ms * 1e-3),
        "newton_its": [rep.its[k] for k in range(rep.ngrids)],
        "reasons": [fg.snes_reason_name(rep.reason[k]) for k in range(rep.ngrids)],
        "inner_its_total": rep.total_ksp_its, "errinf": rep.errinf,
        "grid_ms": [rep.grid_ms[k] for k in range(rep.ngrids)],
        "inner_its_per_grid": [sum(rep.ksp_its[k][i] for i in range(rep.its[k])) for k in range(rep.ngrids)],
    }
    # the same method on the host cores: the oracle's Newton + BiCGStab + Poisson-multigrid
    # solve (FP64, OpenMP) of the same 33^2 -> 1025^2 sequence, best of two
    try:
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import _ms_oracle as mso
        import _oracle as orc
        best = None
        for _ in range(2):
            t0 = time.perf_counter()
            _, nk = mso.nk_solve(base=33, grid_sequence=5, rtol=1e-10)
            dt = time.perf_counter() - t0
            best = dt if best is None or dt < best else best
        m = nk.m[nk.ngrids - 1]
        out["cpu_baseline"] = {"value": m * m / best, "unit": "DOF/s", "cores": orc.lib().or_num_threads(),
                               "kind": "port", "newton_its": [nk.its[k] for k in range(nk.ngrids)],
                               "inner_its_total": nk.ksp_its, "errinf": nk.errinf,
                               "sample": "oracle Newton + BiCGStab/Poisson-MG (FP64, OpenMP), 33^2 -> %d^2 by grid "
                                         "sequencing, snes rtol 1e-10, ksp rtol 1e-5, best of 2 (%.2f s)" % (m, best)}
        out["gpu_over_cpu"] = out["dof_per_s"] / out["cpu_baseline"]["value"]
    except Exception as e:  # oracle library missing: report why
        out["cpu_baseline"] = {"unavailable": str(e)[:200]}
    return out


def clients_leg(fg):
    """The other clients of the Poisson call-backs at 1025^2 (best of 3 solves)."""
    out = {}
    for name, opts, args in (
            ("bratu", fg.bratu_options, "-lb_exact -da_refine 9 -snes_rtol 1e-10"),
            ("obstacle", fg.obstacle_options, "-snes_grid_sequence 9")):
        o = opts(args)
        with fg.MsSolver(o) as s:
            s.solve()
            best = min((s.solve() for _ in range(3)), key=lambda r: r.solve_ms)
        last = best.ngrids - 1
        out[name] = {"options": args, "dofs": best.dofs, "solve_ms": best.solve_ms,
                     "dof_per_s": best.dofs / (best.solve_ms * 1e-3), "newton_its": best.its[last],
                     "inner_its_total": best.total_ksp_its, "errinf": best.errinf,
                     "reason": fg.snes_reason_name(best.reason[last])}
        if name == "obstacle":
            out[name]["active_area_err"] = best.active_area_err
    return out


def serve_leg(fg, n_req, rate=2000.0, workers=16):
    """Mixed 2D/3D serving stream through the continuous-batching server."""
    from p4pdes_gb300 import serve
    stream = serve.make_stream(n_req, rate=rate, seed=2)
    with fg.Server(hbm_budget_bytes=120 << 30, workers=workers, rtol=1e-8) as srv:
        # pre-warm the pool: `workers` resident solvers of every size in the stream
        keys = sorted({(d, n) for _, d, n in stream})
        wstream = [(0.0, d, n) for d, n in keys for _ in range(workers)]
        serve.run_stream(srv, wstream, distinct_rhs=1)
        out = serve.run_stream(srv, stream)
        out["pool"] = srv.stats()
    out["workload"] = ("Poisson arrivals %.0f req/s (seed 2), 2D n in [65,1025] / 3D n in [33,257] log-uniform "
                       "rounded to 2^k+1, f ~ N(0,1), rtol 1e-8 mixed, HBM budget 120 GB, %d workers, "
                       "pinned host arrays" % (rate, workers))
    out["latency"] = "host clock, submit -> solution copied back to the host"
    return out


def run_ours(args):
    import torch
    import p4pdes_gb300 as fg

    world, rank, local = dist_setup()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    stream = torch.cuda.Stream(device=dev)
    W, K = max(3, args.warmup), max(1, args.steps)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    argv = BASE_ARGS.format(r=args.refine).split()
    o_mx = fg.options(argv + ["-fsh_precision", "mixed"])
    o_64 = fg.options(argv)
    N = o_mx.dofs
    f, g = manupoly_fg(torch, o_mx, dev)
    for o in (o_mx, o_64):
        o.ctx.problem, o.ctx.f, o.ctx.g = fg.USER, f.data_ptr(), g.data_ptr()
    u = torch.empty(o_mx.shape, dtype=torch.float64, device=dev)
    info = fg.info_for(o_mx)
    ctx_exact = fg.Ctx.from_buffer_copy(o_mx.ctx)
    ctx_exact.problem = fg.MANUPOLY

    # ---- value: mixed form, inputs resident
    s_mx = fg.Solver(o_mx, stream=stream.cuda_stream)
    for _ in range(W):
        rep = s_mx.solve(u)
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches = 0
    with Clocks(local) as clk:
        e0.record(stream)
        reps = []
        for _ in range(K):
            reps.append(s_mx.solve(u))
        e1.record(stream)
        barrier()
    ms = e0.elapsed_time(e1)
    launches = sum(r.launches for r in reps)
    rep_mx = reps[-1]
    err_mx = fg.error_norms(info, u, ctx_exact)
    value, ms = job_rate(N * K, ms, world, dev)

    # roofline of the dominant kernel: the largest share of the solve's kernel time in the launch
    # list is the FP32 CG direction update fused with the apply (v_cgp_apply) on the 513^3 level;
    # the solve runs it in pairs (y64 left alone, then both owed updates): "cgp_apply_acc_pair"
    # times the pair, one "launch" of the entry below being the two kernels
    rk = args.roofline_kernel
    kms, kbytes = s_mx.time_kernel(rk, 20)
    kernel_table = {}
    for name in ("smooth", "smooth_first", "smooth_dots", "smooth_zero", "cgp_apply", "cgp_apply_acc",
                 "cgp_apply_acc_pair", "cg_update",
                 "resid", "restrict", "resid_restrict", "prolong", "demote", "residual64"):
        try:
            t, b = s_mx.time_kernel(name, 10)
        except fg.FishError:
            continue
        kernel_table[name] = {"ms": t, "algorithmic_bytes": b, "gbs": b / (t * 1e-3) / 1e9}
    if "residual64" in kernel_table:
        # the FP64 residual is bound by the FP64 pipe, not HBM: 3 adds + 4 FMAs
        # (11 flops) per node, against the device's measured FP64 FMA rate
        ent = kernel_table["residual64"]
        peak64 = fg.fp64_fma_rate(5)
        ent.update({"bound": "fp64", "fp64_flops_per_node": 11,
                    "fp64_tflops": 11.0 * N / (ent["ms"] * 1e-3) / 1e12, "fp64_peak_tflops": peak64,
                    "fp64_peak_kind": "measured (independent FMA chains on every SM)"})
        ent["fp64_frac"] = ent["fp64_tflops"] / peak64

    # ---- plain FP64 form beside it
    s_64 = fg.Solver(o_64, stream=stream.cuda_stream)
    s_64.solve(u)
    barrier()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    rep_64 = s_64.solve(u)
    f1.record(stream)
    barrier()
    ms64 = f0.elapsed_time(f1)
    err_64 = fg.error_norms(info, u, ctx_exact)
    s_64.close()

    # ---- e2e: host arrays through the C ABI (f, g in; u out)
    s_mx.close()
    o_e2e = fg.options(argv + ["-fsh_precision", "mixed"])
    o_e2e.ctx.problem = fg.USER
    s_e = fg.Solver(o_e2e, stream=stream.cuda_stream)
    fh = f.cpu().pin_memory()
    gh = g.cpu().pin_memory()
    uh = torch.empty(o_mx.shape, dtype=torch.float64).pin_memory()
    uh2 = torch.empty(o_mx.shape, dtype=torch.float64).pin_memory()
    del f, g
    h2d_bytes = s_e.host_bytes_in(gh)
    for _ in range(1):
        s_e.solve_host(fh, gh, uh)
    s_e.solve_host_many([fh] * 2, [gh] * 2, [uh, uh2])  # warm: staging buffers and copy streams
    barrier()
    # one call per step: f in, solve, u out in sequence
    h0, h1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    h0.record(stream)
    for _ in range(K):
        s_e.solve_host(fh, gh, uh)
    h1.record(stream)
    barrier()
    ms_single = h0.elapsed_time(h1)
    # K steps in one pipelined call (the call returns when every u is in host memory)
    h0.record(stream)
    t0 = time.perf_counter()
    reps_e = s_e.solve_host_many([fh] * K, [gh] * K, [uh if k % 2 == 0 else uh2 for k in range(K)])
    wall_e = (time.perf_counter() - t0) * 1e3
    h1.record(stream)
    barrier()
    ms_e = max(h0.elapsed_time(h1), wall_e)
    assert all(r.reason > 0 for r in reps_e)
    s_e.close()
    e2e, _ = job_rate(N * K, ms_e, world, dev)
    e2e_single, _ = job_rate(N * K, ms_single, world, dev)

    if rank != 0:
        return
    pk, pk_kind = peaks()
    hbm = float(pk.get("hbm_gbs", 6800.0))
    achieved = kbytes / (kms * 1e-3) / 1e9
    traffic = None
    try:
        tr = json.load(open(os.path.join(ROOT, "profiles", "traffic.json")))
        traffic = tr.get(rk, {}).get("dram_bytes_per_launch")
    except Exception:
        pass
    cpu_v, cpu_info = cpu_baseline(args.refine, steps=1)  # one whole solve of the same workload
    batch = batch_leg(torch, fg, args.batch_instances) if args.batch_instances > 0 else None
    serving = serve_leg(fg, args.serve_requests) if args.serve_requests > 0 else None
    if serving is not None:
        # the same stream at a rate one GB300 sustains (the 2000 req/s stream offers about twice its
        # throughput, so its latencies are mostly queueing): latency without a growing queue
        serving["at_sustainable_rate"] = serve_leg(fg, max(200, args.serve_requests // 2), rate=500.0)
    c1 = c1_leg(torch, fg)
    minimal = minimal_leg(fg) if args.minimal else None
    if minimal is not None:
        minimal["other_clients"] = clients_leg(fg)
    line = {
        "metric": METRIC, "value": value, "unit": "DOF/s", "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64", "data": "synthetic (manufactured manupoly problem; f and g sampled at the nodes)",
        "config": {
            "workload": WORKLOAD,
            "form": "mixed = FP32 V-cycle + FP32 inner CG inside FP64 iterative refinement",
            "dofs": N, "levels": o_mx.mg_levels, "parallelism": "replicas" if world > 1 else "1 GPU",
            "l2": "no flush: every vector (1.08 GB FP64) exceeds L2",
            "mixed": {"ms": ms / K, "inner_its": rep_mx.its, "outer_its": rep_mx.outer_its,
                      "inner_its_per_outer": [rep_mx.inner_its[i] for i in range(min(rep_mx.outer_its, 32))],
                      "outer_true_residuals": rep_mx.history(),
                      "true_rel_resid": rep_mx.true_rel_resid, "errinf": err_mx[0], "err2h": err_mx[1]},
            "fp64": {"ms": ms64, "dof_per_s": N / (ms64 * 1e-3), "its": rep_64.its,
                     "true_rel_resid": rep_64.true_rel_resid, "errinf": err_64[0], "err2h": err_64[1]},
            "mixed_over_fp64": (N / (ms / K * 1e-3)) / (N / (ms64 * 1e-3)),
            # like for like against the oracle's FP64 solve of the same workload on the host cores
            "fp64_over_cpu": (N / (ms64 * 1e-3)) / cpu_v,
            "mixed_over_cpu": value / cpu_v,
            "e2e_over_cpu": e2e / cpu_v,
            "error_ratio_mixed_over_fp64": err_mx[0] / err_64[0],
            "batch": batch,
            "serving": serving,
            "minimal": minimal,
            "c1_2d_257": c1,
        },
        "e2e": {"value": e2e, "unit": "DOF/s", "h2d_bytes_per_step": h2d_bytes, "d2h_bytes_per_step": 8 * N,
                "ms_per_step": ms_e / K,
                "note": "K solves through fishgpu_solver_solve_host_many from pinned host arrays: every step's f "
                        "whole in, g only on the boundary (read in place from pinned host memory), u back, the "
                        "copies of steps k+1 / k-1 overlapping the solve of step k",
                "single_calls": {"value": e2e_single, "ms_per_step": ms_single / K,
                                 "note": "one fishgpu_solver_solve_host call per step: f in, solve, u out in "
                                         "sequence"}},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": rk, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": traffic, "peak_kind": pk_kind,
                     "algorithmic_bytes_per_launch": kbytes, "ms_per_launch": kms,
                     "kernels_per_launch": 2 if rk.endswith("_pair") else 1,
                     "fine_level_kernels": {k: dict(v, frac=v["gbs"] / hbm) for k, v in kernel_table.items()}},
        "cpu_baseline": {"value": cpu_v, "unit": "DOF/s", "cores": cpu_info["cores"], "kind": "port",
                         "sample": cpu_info["sample"]},
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--refine", type=int, default=8, help="-da_refine (8: 513^3)")
    ap.add_argument("--roofline-kernel", default="cgp_apply_acc_pair")
    ap.add_argument("--batch-instances", type=int, default=4096, help="batched 2D leg (0: skip)")
    ap.add_argument("--serve-requests", type=int, default=1000, help="serving-stream leg (0: skip)")
    ap.add_argument("--minimal", type=int, default=1, help="minimal-surface leg (0: skip)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
