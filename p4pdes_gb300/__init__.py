"""p4pdes_gb300 -- GB300 (sm_103a) solver for the fish.c / poissonfunctions.c path.

Python front end of libfishgpu.so (the C ABI declared in include/fishgpu.h).
It mirrors the reference's interface for this path:

  * ``Poisson{1,2,3}DFunctionLocal(info, au, aF, user)``  -- residual call-backs
    (c/ch6/poissonfunctions.c:4-115), same argument meaning, arrays are CUDA
    tensors indexed with global (i,j,k) like the DMDA arrays;
  * ``Poisson{1,2,3}DOperatorApply(info, p, q, user)``   -- the Jacobian of
    c/ch6/poissonfunctions.c:117-258 applied matrix-free, returns p.q;
  * ``FormUExact``, ``InitialState``, ``error_norms``     -- c/ch6/fish.c:237-340,
    c/ch6/poissonfunctions.c:260-346;
  * ``options(argv)`` parses fish's flags (-fsh_*, -da_refine, -ksp_*, -pc_*,
    -mg_levels_*), ``solve(opts)`` runs the fish flow on the GPU;
  * ``Solver`` keeps one hierarchy device-resident, ``Batch`` solves many 2D
    instances together, ``Server`` admits a stream of solves by HBM budget.

Errors raise FishError carrying the library status (the reference returns
PetscErrorCode).  There is no CPU fallback: if the library is missing the
import of any entry point raises.
"""
import ctypes
import os

__all__ = [
    "Info", "Ctx", "Opts", "Report", "FishError", "load", "options", "info_for", "solve",
    "Poisson1DFunctionLocal", "Poisson2DFunctionLocal", "Poisson3DFunctionLocal",
    "Poisson1DOperatorApply", "Poisson2DOperatorApply", "Poisson3DOperatorApply",
    "FormUExact", "InitialState", "error_norms", "reason_name",
    "Solver", "Batch", "Server", "estimate_bytes", "server_request_opts",
    "MsSolver", "ms_options", "ms_solve", "MinimalFunctionLocal", "snes_reason_name",
    "bratu_options", "BratuFunctionLocal", "obstacle_options",
]

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib", "libfishgpu.so")

MANUPOLY, MANUEXP, ZERO, USER = 0, 1, 2, 3
PROBLEMS = {"manupoly": MANUPOLY, "manuexp": MANUEXP, "zero": ZERO}
PC_NONE, PC_JACOBI, PC_MG = 0, 1, 2
SMOOTH_CHEBYSHEV, SMOOTH_RICHARDSON = 0, 1
NORM_PRECONDITIONED, NORM_UNPRECONDITIONED = 0, 1
FP64, MIXED = 0, 1
INITIAL_ZEROS, INITIAL_RANDOM, INITIAL_GIVEN = 0, 1, 2
MAX_HIST = 512
MAX_OUTER = 32

c_int, c_double, c_void_p, c_ll, c_ull = (ctypes.c_int, ctypes.c_double, ctypes.c_void_p,
                                          ctypes.c_longlong, ctypes.c_ulonglong)


class Info(ctypes.Structure):
    """fishgpu_info: the DMDALocalInfo fields plus the bounding box."""
    _fields_ = [("dim", c_int), ("mx", c_int), ("my", c_int), ("mz", c_int),
                ("xs", c_int), ("ys", c_int), ("zs", c_int),
                ("xm", c_int), ("ym", c_int), ("zm", c_int),
                ("xmin", c_double * 3), ("xmax", c_double * 3)]


class Ctx(ctypes.Structure):
    """fishgpu_ctx: PoissonCtx with a problem enum in place of f_rhs/g_bdry."""
    _fields_ = [("Lx", c_double), ("Ly", c_double), ("Lz", c_double),
                ("cx", c_double), ("cy", c_double), ("cz", c_double),
                ("problem", c_int), ("dim", c_int), ("f", c_void_p), ("g", c_void_p)]


class Opts(ctypes.Structure):
    _fields_ = [("ctx", Ctx), ("mx", c_int), ("my", c_int), ("mz", c_int), ("da_refine", c_int),
                ("initial_type", c_int), ("initial_gonboundary", c_int), ("seed", c_ull),
                ("rtol", c_double), ("atol", c_double), ("dtol", c_double),
                ("max_it", c_int), ("norm_type", c_int), ("pc_type", c_int), ("mg_levels", c_int),
                ("mg_cycles", c_int), ("smooth_type", c_int), ("smooth_its", c_int),
                ("esteig", c_double * 4), ("richardson_scale", c_double), ("precision", c_int),
                ("inner_rtol", c_double), ("inner_max_it", c_int), ("outer_max_it", c_int),
                ("graph_iters", c_int), ("monitor", c_int), ("converged_reason", c_int),
                ("snes_monitor", c_int), ("fuse_smooth", c_int), ("device_loop", c_int), ("loop_cap", c_int),
                ("first_floor_scale", c_double), ("inner_accurate", c_int), ("fuse_restrict", c_int),
                ("tma_apply", c_int), ("vtail", c_int),
                ("vtail_points", c_int), ("persist", c_int), ("persist_points", c_int),
                ("persist_tail", c_int), ("fuse_cgr", c_int), ("coop_tail", c_int), ("pair_y", c_int)]

    @property
    def dofs(self):
        d = self.ctx.dim
        return self.mx * (self.my if d >= 2 else 1) * (self.mz if d >= 3 else 1)

    @property
    def shape(self):
        """(mz, my, mx) of the dense array, x fastest."""
        d = self.ctx.dim
        return (self.mz if d >= 3 else 1, self.my if d >= 2 else 1, self.mx)


class Report(ctypes.Structure):
    _fields_ = [("its", c_int), ("reason", c_int), ("outer_its", c_int), ("nhist", c_int),
                ("hist", c_double * MAX_HIST), ("fnorm0", c_double), ("fnorm1", c_double),
                ("errinf", c_double), ("err2h", c_double), ("true_rel_resid", c_double),
                ("setup_ms", c_double), ("solve_ms", c_double), ("dofs", c_ll), ("launches", c_ll),
                ("inner_its", c_int * MAX_OUTER)]

    def history(self):
        return [self.hist[i] for i in range(min(self.nhist, MAX_HIST))]


class BatchOpts(ctypes.Structure):
    _fields_ = [("rtol", c_double), ("atol", c_double), ("inner_rtol", c_double), ("inner_max_it", c_int),
                ("outer_max_it", c_int), ("smooth_its", c_int), ("mg_cycles", c_int), ("esteig", c_double * 4),
                ("tune", c_int), ("inner_accurate", c_int), ("tune_sweeps", c_int)]


class BatchReport(ctypes.Structure):
    _fields_ = [("ninst", c_int), ("groups", c_int), ("converged", c_int), ("max_outer", c_int),
                ("max_inner", c_int), ("total_inner_its", c_ll), ("dofs", c_ll), ("launches", c_ll),
                ("solve_ms", c_double)]


class ServerOpts(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", c_ll), ("workers", c_int), ("rtol", c_double), ("precision", c_int),
                ("fifo", c_int), ("batch_max", c_int)]


class ServerResult(ctypes.Structure):
    _fields_ = [("status", c_int), ("its", c_int), ("outer_its", c_int), ("rel_resid", c_double),
                ("queue_ms", c_double), ("service_ms", c_double), ("latency_ms", c_double)]


MS_TENT, MS_CATENOID = 0, 1
MS_MAX_GRIDS, MS_MAX_ITS = 12, 64


NL_MINIMAL, NL_BRATU, NL_OBSTACLE = 0, 1, 2
BRATU_ZERO, BRATU_LIOUVILLE = 0, 1


class MsCtx(ctypes.Structure):
    _fields_ = [("problem", c_int), ("q", c_double), ("catenoid_c", c_double), ("tent_H", c_double),
                ("model", c_int), ("lam", c_double)]


class MsOpts(ctypes.Structure):
    _fields_ = [("ctx", MsCtx), ("mx", c_int), ("my", c_int), ("grid_sequence", c_int), ("exact_init", c_int),
                ("rtol", c_double), ("atol", c_double), ("stol", c_double), ("max_it", c_int),
                ("line_search", c_int), ("ksp_rtol", c_double), ("ksp_max_it", c_int), ("pc_type", c_int),
                ("mg_levels", c_int), ("monitor_degree", c_int), ("snes_monitor", c_int),
                ("converged_reason", c_int), ("ksp_converged_reason", c_int), ("loop_cap", c_int),
                ("inner_block", c_int), ("inner_persist", c_int), ("vtail_points", c_int)]


class MsReport(ctypes.Structure):
    _fields_ = [("ngrids", c_int), ("m", c_int * MS_MAX_GRIDS), ("its", c_int * MS_MAX_GRIDS),
                ("reason", c_int * MS_MAX_GRIDS), ("ksp_its", (c_int * MS_MAX_ITS) * MS_MAX_GRIDS),
                ("ksp_reason", (c_int * MS_MAX_ITS) * MS_MAX_GRIDS),
                ("fnorm", (c_double * (MS_MAX_ITS + 1)) * MS_MAX_GRIDS),
                ("area", ((c_double * 3) * (MS_MAX_ITS + 1)) * MS_MAX_GRIDS),
                ("errinf", c_double), ("solve_ms", c_double), ("dofs", c_ll), ("total_ksp_its", c_ll),
                ("nfuncs", c_ll), ("grid_ms", c_double * MS_MAX_GRIDS), ("err1", c_double),
                ("active_area_err", c_double), ("n_active", c_ll), ("inner_form", c_int * MS_MAX_GRIDS)]

    def fnorms(self, k):
        return [self.fnorm[k][i] for i in range(self.its[k] + 1)]

    def areas(self, k):
        return [tuple(self.area[k][i]) for i in range(self.its[k] + 1)]


class FishError(RuntimeError):
    def __init__(self, code, what=""):
        self.code = code
        msg = load().fishgpu_strerror(code).decode() if _lib is not None else str(code)
        super().__init__("%s: %s (status %d)" % (what, msg, code) if what else msg)


_lib = None
_P = ctypes.POINTER


def load():
    """Load libfishgpu.so (built in-tree by p4pdes_gb300.build)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libfishgpu.so is not built (%s); run p4pdes_gb300.build.build()" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for dim in (1, 2, 3):
        f = getattr(lib, "Poisson%dDFunctionLocal_gpu" % dim)
        f.argtypes = [_P(Info), c_void_p, c_void_p, _P(Ctx), c_void_p]
        f.restype = c_int
        f = getattr(lib, "Poisson%dDOperatorApply_gpu" % dim)
        f.argtypes = [_P(Info), c_void_p, c_void_p, c_void_p, _P(Ctx), c_void_p]
        f.restype = c_int
    lib.PoissonOperatorApplyNoAlloc_gpu.argtypes = [_P(Info), c_void_p, c_void_p, c_void_p, _P(Ctx), c_void_p]
    lib.PoissonOperatorApplyNoAlloc_gpu.restype = c_int
    lib.FormUExact_gpu.argtypes = [_P(Info), c_void_p, _P(Ctx), c_void_p]
    lib.InitialState_gpu.argtypes = [_P(Info), c_int, c_int, c_ull, c_void_p, _P(Ctx), c_void_p]
    lib.ErrorNorms_gpu.argtypes = [_P(Info), c_void_p, _P(Ctx), _P(c_double), _P(c_double), c_void_p]
    lib.fishgpu_strerror.argtypes = [c_int]
    lib.fishgpu_strerror.restype = ctypes.c_char_p
    lib.fishgpu_reason_name.argtypes = [c_int]
    lib.fishgpu_reason_name.restype = ctypes.c_char_p
    lib.fishgpu_opts_default.argtypes = [_P(Opts)]
    lib.fishgpu_opts_parse.argtypes = [_P(Opts), c_int, _P(ctypes.c_char_p)]
    lib.fishgpu_solver_create.argtypes = [_P(Opts), c_void_p, _P(c_void_p)]
    lib.fishgpu_solver_solve.argtypes = [c_void_p, c_void_p, _P(Report)]
    lib.fishgpu_solver_destroy.argtypes = [c_void_p]
    lib.fishgpu_solver_bytes.argtypes = [c_void_p]
    lib.fishgpu_solver_bytes.restype = c_ll
    lib.fishgpu_solve.argtypes = [_P(Opts), c_void_p, _P(Report)]
    lib.fishgpu_solve_host.argtypes = [_P(Opts), c_void_p, c_void_p, c_void_p, _P(Report)]
    lib.fishgpu_solver_solve_host.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, _P(Report)]
    lib.fishgpu_solver_solve_host.restype = c_int
    lib.fishgpu_solver_solve_host_many.argtypes = [c_void_p, c_int, _P(c_void_p), _P(c_void_p), _P(c_void_p),
                                                   _P(Report)]
    lib.fishgpu_solver_solve_host_many.restype = c_int
    lib.fishgpu_batch_opts_default.argtypes = [_P(BatchOpts)]
    lib.fishgpu_batch_create.argtypes = [_P(BatchOpts), c_int, _P(c_int), _P(c_void_p)]
    lib.fishgpu_batch_solve.argtypes = [c_void_p, _P(c_void_p), _P(c_void_p), _P(BatchReport)]
    lib.fishgpu_batch_results.argtypes = [c_void_p, _P(c_int), _P(c_int), _P(c_double), _P(c_int)]
    lib.fishgpu_batch_destroy.argtypes = [c_void_p]
    lib.fishgpu_batch_groups.argtypes = [c_void_p, _P(c_int), _P(c_int), _P(c_int)]
    for name in ("fishgpu_batch_opts_default", "fishgpu_batch_create", "fishgpu_batch_solve",
                 "fishgpu_batch_results", "fishgpu_batch_destroy", "fishgpu_batch_groups"):
        getattr(lib, name).restype = c_int
    lib.fishgpu_group_create.argtypes = [_P(BatchOpts), c_int, c_int, _P(c_void_p)]
    lib.fishgpu_group_create.restype = c_int
    lib.fishgpu_group_bytes.argtypes = [c_void_p]
    lib.fishgpu_group_bytes.restype = c_ll
    lib.fishgpu_group_solve_host.argtypes = [c_void_p, c_int, _P(c_void_p), _P(c_void_p), _P(c_int), _P(c_int),
                                             _P(c_double)]
    lib.fishgpu_group_solve_host.restype = c_int
    lib.fishgpu_group_destroy.argtypes = [c_void_p]
    lib.fishgpu_group_destroy.restype = c_int
    lib.fishgpu_solver_time_kernel.argtypes = [c_void_p, ctypes.c_char_p, c_int, _P(c_double), _P(c_double)]
    lib.fishgpu_fp64_fma_rate.argtypes = [c_int, _P(c_double)]
    lib.fishgpu_fp64_fma_rate.restype = c_int
    lib.fishgpu_ms_opts_default.argtypes = [_P(MsOpts)]
    lib.fishgpu_bratu_opts_default.argtypes = [_P(MsOpts)]
    lib.fishgpu_bratu_opts_default.restype = c_int
    lib.fishgpu_obstacle_opts_default.argtypes = [_P(MsOpts)]
    lib.fishgpu_obstacle_opts_default.restype = c_int
    lib.BratuFunctionLocal_gpu.argtypes = [_P(Info), c_void_p, c_void_p, c_double, c_int, c_void_p]
    lib.BratuFunctionLocal_gpu.restype = c_int
    lib.fishgpu_ms_opts_parse.argtypes = [_P(MsOpts), c_int, _P(ctypes.c_char_p)]
    lib.fishgpu_ms_solver_create.argtypes = [_P(MsOpts), c_void_p, _P(c_void_p)]
    lib.fishgpu_ms_solver_solve.argtypes = [c_void_p, c_void_p, _P(MsReport)]
    lib.fishgpu_ms_solver_destroy.argtypes = [c_void_p]
    lib.fishgpu_ms_solve.argtypes = [_P(MsOpts), c_void_p, _P(MsReport)]
    lib.MinimalFunctionLocal_gpu.argtypes = [_P(Info), c_void_p, c_void_p, _P(MsCtx), c_void_p]
    lib.fishgpu_snes_reason_name.argtypes = [c_int]
    lib.fishgpu_snes_reason_name.restype = ctypes.c_char_p
    for name in ("fishgpu_ms_opts_default", "fishgpu_ms_opts_parse", "fishgpu_ms_solver_create",
                 "fishgpu_ms_solver_solve", "fishgpu_ms_solver_destroy", "fishgpu_ms_solve",
                 "MinimalFunctionLocal_gpu"):
        getattr(lib, name).restype = c_int
    lib.fishgpu_petsc_vec_write.argtypes = [ctypes.c_char_p, c_int, c_void_p, c_ll]
    lib.fishgpu_petsc_vec_read.argtypes = [ctypes.c_char_p, c_int, c_void_p, c_ll, _P(c_ll)]
    lib.fishgpu_petsc_mat_write_aij.argtypes = [ctypes.c_char_p, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p]
    lib.fishgpu_petsc_mat_read_aij.argtypes = [ctypes.c_char_p, c_int, _P(c_int), _P(c_int), _P(c_ll), c_void_p,
                                               c_void_p, c_void_p]
    for name in ("fishgpu_petsc_vec_write", "fishgpu_petsc_vec_read", "fishgpu_petsc_mat_write_aij",
                 "fishgpu_petsc_mat_read_aij"):
        getattr(lib, name).restype = c_int
    lib.fishgpu_solver_host_bytes_in.argtypes = [c_void_p, c_void_p]
    lib.fishgpu_solver_host_bytes_in.restype = c_ll
    lib.fishgpu_solver_estimate_bytes.argtypes = [_P(Opts)]
    lib.fishgpu_solver_estimate_bytes.restype = c_ll
    lib.fishgpu_server_opts_default.argtypes = [_P(ServerOpts)]
    lib.fishgpu_server_create.argtypes = [_P(ServerOpts), _P(c_void_p)]
    lib.fishgpu_server_submit.argtypes = [c_void_p, c_int, c_int, c_void_p, c_void_p, _P(c_ll)]
    lib.fishgpu_server_wait.argtypes = [c_void_p, c_ll, c_double, _P(ServerResult)]
    lib.fishgpu_server_stats.argtypes = [c_void_p, _P(c_ll), _P(c_int), _P(c_ll), _P(c_ll)]
    lib.fishgpu_server_group_stats.argtypes = [c_void_p, _P(c_ll), _P(c_ll)]
    lib.fishgpu_solver_barrier_selftest.argtypes = [c_void_p, c_int]
    lib.fishgpu_solver_barrier_selftest.restype = c_int
    lib.fishgpu_server_group_stats.restype = c_int
    lib.fishgpu_server_destroy.argtypes = [c_void_p]
    for name in ("fishgpu_server_opts_default", "fishgpu_server_create", "fishgpu_server_submit",
                 "fishgpu_server_wait", "fishgpu_server_stats", "fishgpu_server_destroy"):
        getattr(lib, name).restype = c_int
    for name in ("FormUExact_gpu", "InitialState_gpu", "ErrorNorms_gpu", "fishgpu_opts_default",
                 "fishgpu_opts_parse", "fishgpu_solver_create", "fishgpu_solver_solve",
                 "fishgpu_solver_destroy", "fishgpu_solve", "fishgpu_solve_host",
                 "fishgpu_solver_time_kernel"):
        getattr(lib, name).restype = c_int
    _lib = lib
    return lib


def _check(rc, what):
    if rc != 0:
        raise FishError(rc, what)


def reason_name(reason):
    return load().fishgpu_reason_name(reason).decode()


def options(argv=()):
    """fishgpu_opts from fish's command-line flags (a list or a string)."""
    if isinstance(argv, str):
        argv = argv.split()
    o = Opts()
    lib = load()
    _check(lib.fishgpu_opts_default(ctypes.byref(o)), "fishgpu_opts_default")
    arr = (ctypes.c_char_p * max(1, len(argv)))(*[a.encode() for a in argv])
    _check(lib.fishgpu_opts_parse(ctypes.byref(o), len(argv), arr), "fishgpu_opts_parse")
    return o


def info_for(opts):
    """The whole-grid local info of one GPU holding the whole DMDA."""
    d = opts.ctx.dim
    inf = Info()
    inf.dim = d
    inf.mx = opts.mx
    inf.my = opts.my if d >= 2 else 1
    inf.mz = opts.mz if d >= 3 else 1
    inf.xm, inf.ym, inf.zm = inf.mx, inf.my, inf.mz
    inf.xmax[0], inf.xmax[1], inf.xmax[2] = opts.ctx.Lx, opts.ctx.Ly, opts.ctx.Lz
    return inf


def _ptr(t):
    if t is None:
        return None
    if not t.is_cuda or not t.is_contiguous():
        raise ValueError("expected a contiguous CUDA tensor")
    return t.data_ptr()


def _stream(stream):
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    return int(stream)


def _fl(dim, info, au, aF, user, stream):
    fn = getattr(load(), "Poisson%dDFunctionLocal_gpu" % dim)
    _check(fn(ctypes.byref(info), _ptr(au), _ptr(aF), ctypes.byref(user), _stream(stream)),
           "Poisson%dDFunctionLocal" % dim)


def Poisson1DFunctionLocal(info, au, aF, user, stream=None):
    _fl(1, info, au, aF, user, stream)


def Poisson2DFunctionLocal(info, au, aF, user, stream=None):
    _fl(2, info, au, aF, user, stream)


def Poisson3DFunctionLocal(info, au, aF, user, stream=None):
    _fl(3, info, au, aF, user, stream)


def _apply(dim, info, p, q, user, stream, dot):
    import torch
    fn = getattr(load(), "Poisson%dDOperatorApply_gpu" % dim)
    d = torch.zeros(1, dtype=torch.float64, device=p.device) if dot else None
    _check(fn(ctypes.byref(info), _ptr(p), _ptr(q), _ptr(d), ctypes.byref(user), _stream(stream)),
           "Poisson%dDOperatorApply" % dim)
    return d


def Poisson1DOperatorApply(info, p, q, user, stream=None, dot=True):
    return _apply(1, info, p, q, user, stream, dot)


def Poisson2DOperatorApply(info, p, q, user, stream=None, dot=True):
    return _apply(2, info, p, q, user, stream, dot)


def Poisson3DOperatorApply(info, p, q, user, stream=None, dot=True):
    return _apply(3, info, p, q, user, stream, dot)


def FormUExact(info, u, user, stream=None):
    _check(load().FormUExact_gpu(ctypes.byref(info), _ptr(u), ctypes.byref(user), _stream(stream)),
           "FormUExact")


def InitialState(info, initial_type, gbdry, u, user, seed=0, stream=None):
    _check(load().InitialState_gpu(ctypes.byref(info), initial_type, int(bool(gbdry)), seed, _ptr(u),
                                   ctypes.byref(user), _stream(stream)), "InitialState")


def error_norms(info, u, user, stream=None):
    a, b = c_double(), c_double()
    _check(load().ErrorNorms_gpu(ctypes.byref(info), _ptr(u), ctypes.byref(user), ctypes.byref(a),
                                 ctypes.byref(b), _stream(stream)), "ErrorNorms")
    return a.value, b.value


class Solver:
    """Device-resident hierarchy; solve() runs the fish flow (u0, F(u0), KSP, u)."""

    def __init__(self, opts, stream=None):
        self.opts = opts
        self._h = c_void_p()
        st = None if stream is None else int(stream)
        _check(load().fishgpu_solver_create(ctypes.byref(opts), st, ctypes.byref(self._h)),
               "fishgpu_solver_create")

    def solve(self, u):
        rep = Report()
        rc = load().fishgpu_solver_solve(self._h, _ptr(u), ctypes.byref(rep))
        if rc not in (0, 4):
            raise FishError(rc, "fishgpu_solver_solve")
        return rep

    def solve_host(self, f=None, g=None, u=None):
        """Host-array solve (numpy or pinned torch CPU tensors, float64)."""
        def addr(a):
            if a is None:
                return None
            return a.data_ptr() if hasattr(a, "data_ptr") else a.ctypes.data
        rep = Report()
        rc = load().fishgpu_solver_solve_host(self._h, addr(f), addr(g), addr(u), ctypes.byref(rep))
        if rc not in (0, 4):
            raise FishError(rc, "fishgpu_solver_solve_host")
        return rep

    def solve_host_many(self, fs, gs, us):
        """Host-array solves of len(fs) problems in order, copies overlapped with the
        solves (fishgpu_solver_solve_host_many); gs may be None.  Returns the reports."""
        def addr(a):
            if a is None:
                return None
            return a.data_ptr() if hasattr(a, "data_ptr") else a.ctypes.data
        n = len(fs)
        if len(us) != n or (gs is not None and len(gs) != n):
            raise ValueError("fs, gs and us differ in length")
        arr = lambda xs: (c_void_p * max(1, n))(*[addr(x) for x in xs])
        reps = (Report * max(1, n))()
        rc = load().fishgpu_solver_solve_host_many(self._h, n, arr(fs), None if gs is None else arr(gs), arr(us),
                                                   reps)
        if rc not in (0, 4):
            raise FishError(rc, "fishgpu_solver_solve_host_many")
        return [reps[k] for k in range(n)]

    def barrier_selftest(self, missing):
        """The persistent solve's grid barrier with block 0 absent (missing) or not: the status."""
        return load().fishgpu_solver_barrier_selftest(self._h, int(missing))

    def host_bytes_in(self, g=None):
        """Bytes solve_host moves to the device for f and g."""
        ga = None if g is None else (g.data_ptr() if hasattr(g, "data_ptr") else g.ctypes.data)
        return load().fishgpu_solver_host_bytes_in(self._h, ga)

    def time_kernel(self, name, reps):
        ms, by = c_double(), c_double()
        _check(load().fishgpu_solver_time_kernel(self._h, name.encode(), reps, ctypes.byref(ms),
                                                 ctypes.byref(by)), "time_kernel")
        return ms.value, by.value

    @property
    def device_bytes(self):
        return load().fishgpu_solver_bytes(self._h)

    def close(self):
        if self._h:
            load().fishgpu_solver_destroy(self._h)
            self._h = c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many independent 2D problems -Laplace(u) = f, u = 0 on the boundary of the
    unit square, n x n nodes (n = 2^k + 1), solved together (mixed form)."""

    def __init__(self, sizes, rtol=1e-8, tune=True, **kw):
        o = BatchOpts()
        _check(load().fishgpu_batch_opts_default(ctypes.byref(o)), "fishgpu_batch_opts_default")
        o.rtol = rtol
        o.tune = int(bool(tune))
        for k, v in kw.items():
            setattr(o, k, v)
        self.sizes = [int(n) for n in sizes]
        arr = (c_int * len(self.sizes))(*self.sizes)
        self._h = c_void_p()
        _check(load().fishgpu_batch_create(ctypes.byref(o), len(self.sizes), arr, ctypes.byref(self._h)),
               "fishgpu_batch_create")

    def solve(self, fs, us):
        """fs, us: lists of contiguous CUDA float64 tensors (n, n)."""
        n = len(self.sizes)
        fa = (c_void_p * n)(*[_ptr(f) for f in fs])
        ua = (c_void_p * n)(*[_ptr(u) for u in us])
        rep = BatchReport()
        rc = load().fishgpu_batch_solve(self._h, fa, ua, ctypes.byref(rep))
        if rc not in (0, 4):
            raise FishError(rc, "fishgpu_batch_solve")
        return rep

    def results(self):
        n = len(self.sizes)
        a, b, c, d = (c_int * n)(), (c_int * n)(), (c_double * n)(), (c_int * n)()
        _check(load().fishgpu_batch_results(self._h, a, b, c, d), "fishgpu_batch_results")
        return list(a), list(b), list(c), list(d)

    def groups(self):
        """[(n, instances, smoothing steps per level)] per size group, largest first."""
        k = len(set(self.sizes))
        a, b, c = (c_int * k)(), (c_int * k)(), (c_int * k)()
        ng = load().fishgpu_batch_groups(self._h, a, b, c)
        return [(a[g], b[g], c[g]) for g in range(ng)]

    def close(self):
        if self._h:
            load().fishgpu_batch_destroy(self._h)
            self._h = c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Group:
    """`count` same-size 2D problems (n x n, n = 2^k + 1) solved together with the
    batch's kernels on one stream; solve_host takes up to `count` host arrays
    (the rest of the group is empty).  An instance's result does not depend on
    the group it is solved in (tune = 0)."""

    def __init__(self, n, count, rtol=1e-8, **kw):
        o = BatchOpts()
        _check(load().fishgpu_batch_opts_default(ctypes.byref(o)), "fishgpu_batch_opts_default")
        o.rtol = rtol
        o.tune = 0
        o.tune_sweeps = 0
        for k, v in kw.items():
            setattr(o, k, v)
        self.n, self.count = int(n), int(count)
        self._h = c_void_p()
        _check(load().fishgpu_group_create(ctypes.byref(o), self.n, self.count, ctypes.byref(self._h)),
               "fishgpu_group_create")

    @property
    def device_bytes(self):
        return load().fishgpu_group_bytes(self._h)

    def solve_host(self, fs, us):
        """fs, us: host float64 arrays (n, n); returns [(its, outer_its, rel_resid)] per instance."""
        k = len(fs)
        fa = (c_void_p * k)(*[_host_addr(f) for f in fs])
        ua = (c_void_p * k)(*[_host_addr(u) for u in us])
        its, outer, rel = (c_int * k)(), (c_int * k)(), (c_double * k)()
        _check(load().fishgpu_group_solve_host(self._h, k, fa, ua, its, outer, rel), "fishgpu_group_solve_host")
        return [(its[q], outer[q], rel[q]) for q in range(k)]

    def close(self):
        if self._h:
            load().fishgpu_group_destroy(self._h)
            self._h = c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def fp64_fma_rate(reps=5):
    """FP64 FMA throughput of the current device in TFLOP/s (FMA = 2 flops)."""
    t = c_double()
    _check(load().fishgpu_fp64_fma_rate(reps, ctypes.byref(t)), "fp64_fma_rate")
    return t.value


def estimate_bytes(opts):
    """Device bytes a Solver for these options holds (-1: invalid options)."""
    return load().fishgpu_solver_estimate_bytes(ctypes.byref(opts))


def _host_addr(a):
    return a.data_ptr() if hasattr(a, "data_ptr") else a.ctypes.data


class Server:
    """Solve server with continuous batching: requests -Laplace(u) = f on the
    unit square/cube, u = 0 on the boundary, n nodes per side (2^k + 1), are
    admitted as worker slots and HBM budget free up and overlap on the device.
    f and u are host float64 arrays (numpy or CPU tensors, pinned for speed)
    that must stay alive until wait() returns."""

    def __init__(self, hbm_budget_bytes=120 << 30, workers=8, rtol=1e-8, precision=MIXED, fifo=False,
                 batch_max=16):
        o = ServerOpts()
        _check(load().fishgpu_server_opts_default(ctypes.byref(o)), "fishgpu_server_opts_default")
        o.hbm_budget_bytes = int(hbm_budget_bytes)
        o.workers = int(workers)
        o.rtol = rtol
        o.precision = precision
        o.fifo = int(bool(fifo))
        o.batch_max = int(batch_max)
        self._h = c_void_p()
        self._keep = {}
        _check(load().fishgpu_server_create(ctypes.byref(o), ctypes.byref(self._h)), "fishgpu_server_create")

    def submit(self, dim, n, f, u):
        t = c_ll()
        _check(load().fishgpu_server_submit(self._h, dim, n, _host_addr(f), _host_addr(u), ctypes.byref(t)),
               "fishgpu_server_submit")
        self._keep[t.value] = (f, u)
        return t.value

    def wait(self, ticket, timeout_ms=-1.0):
        r = ServerResult()
        _check(load().fishgpu_server_wait(self._h, ticket, timeout_ms, ctypes.byref(r)), "fishgpu_server_wait")
        self._keep.pop(ticket, None)
        return r

    def stats(self):
        b, n, c, e = c_ll(), c_int(), c_ll(), c_ll()
        _check(load().fishgpu_server_stats(self._h, ctypes.byref(b), ctypes.byref(n), ctypes.byref(c),
                                           ctypes.byref(e)), "fishgpu_server_stats")
        gs, gr = c_ll(), c_ll()
        _check(load().fishgpu_server_group_stats(self._h, ctypes.byref(gs), ctypes.byref(gr)),
               "fishgpu_server_group_stats")
        return {"pooled_bytes": b.value, "pooled_solvers": n.value, "created": c.value, "evicted": e.value,
                "group_solves": gs.value, "grouped_requests": gr.value}

    def close(self):
        if self._h:
            load().fishgpu_server_destroy(self._h)
            self._h = c_void_p()
            self._keep.clear()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def server_request_opts(dim, n, rtol=1e-8, precision=MIXED):
    """The solver options the server uses for a (dim, n) request."""
    o = options([])
    o.ctx.dim = dim
    o.ctx.problem = USER
    o.mx = n
    o.my = n if dim >= 2 else 1
    o.mz = n if dim >= 3 else 1
    levels, m = 1, n
    while m > 3 and (m - 1) % 2 == 0:
        m = (m - 1) // 2 + 1
        levels += 1
    o.mg_levels = levels
    o.pc_type = PC_MG
    o.precision = precision
    o.rtol = rtol
    o.norm_type = NORM_UNPRECONDITIONED
    o.persist = 0
    o.coop_tail = 0
    return o


def ms_options(argv=()):
    """Parse minimal.c's flags into an MsOpts."""
    if isinstance(argv, str):
        argv = argv.split()
    o = MsOpts()
    _check(load().fishgpu_ms_opts_default(ctypes.byref(o)), "fishgpu_ms_opts_default")
    arr = (ctypes.c_char_p * max(1, len(argv)))(*[a.encode() for a in argv])
    _check(load().fishgpu_ms_opts_parse(ctypes.byref(o), len(argv), arr), "fishgpu_ms_opts_parse")
    return o


def bratu_options(argv=()):
    """Parse bratu2D.c's flags (-lb_lambda, -lb_exact, -da_refine, -snes_*) into an MsOpts."""
    if isinstance(argv, str):
        argv = argv.split()
    o = MsOpts()
    _check(load().fishgpu_bratu_opts_default(ctypes.byref(o)), "fishgpu_bratu_opts_default")
    arr = (ctypes.c_char_p * max(1, len(argv)))(*[a.encode() for a in argv])
    _check(load().fishgpu_ms_opts_parse(ctypes.byref(o), len(argv), arr), "fishgpu_ms_opts_parse")
    return o


def obstacle_options(argv=()):
    """Parse obstacle.c's flags (-da_refine, -snes_grid_sequence, -snes_*, -ksp_rtol) into an MsOpts."""
    if isinstance(argv, str):
        argv = argv.split()
    o = MsOpts()
    _check(load().fishgpu_obstacle_opts_default(ctypes.byref(o)), "fishgpu_obstacle_opts_default")
    arr = (ctypes.c_char_p * max(1, len(argv)))(*[a.encode() for a in argv])
    _check(load().fishgpu_ms_opts_parse(ctypes.byref(o), len(argv), arr), "fishgpu_ms_opts_parse")
    return o


def BratuFunctionLocal(info, au, aF, lam=1.0, liouville=False, stream=None):
    """FormFunctionLocal of c/ch7/solns/bratu2D.c:188-217 on the device."""
    _check(load().BratuFunctionLocal_gpu(ctypes.byref(info), _ptr(au), _ptr(aF), lam, int(liouville),
                                         _stream(stream)), "BratuFunctionLocal_gpu")


def snes_reason_name(reason):
    return load().fishgpu_snes_reason_name(reason).decode()


class MsSolver:
    """Minimal-surface Newton solver (every grid of the sequence set up once)."""

    def __init__(self, opts, stream=None):
        self.opts = opts
        self._h = c_void_p()
        _check(load().fishgpu_ms_solver_create(ctypes.byref(opts), None if stream is None else int(stream),
                                               ctypes.byref(self._h)), "fishgpu_ms_solver_create")

    def solve(self, u=None):
        """Returns the report; u: optional host float64 array (my, mx) of the last grid."""
        rep = MsReport()
        rc = load().fishgpu_ms_solver_solve(self._h, None if u is None else _host_addr(u), ctypes.byref(rep))
        if rc not in (0, 4):
            raise FishError(rc, "fishgpu_ms_solver_solve")
        return rep

    def close(self):
        if self._h:
            load().fishgpu_ms_solver_destroy(self._h)
            self._h = c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def ms_solve(opts):
    """minimal.c's flow; returns (u (numpy, last grid), report)."""
    import numpy as np
    with MsSolver(opts) as s:
        m = opts.mx
        my = opts.my
        for _ in range(opts.grid_sequence):
            m, my = 2 * m - 1, 2 * my - 1
        u = np.empty((my, m))
        rep = s.solve(u)
    return u, rep


def MinimalFunctionLocal(info, au, aF, ctx, stream=None):
    """FormFunctionLocal of c/ch7/minimal.c:210-282 on the device."""
    _check(load().MinimalFunctionLocal_gpu(ctypes.byref(info), _ptr(au), _ptr(aF), ctypes.byref(ctx),
                                           _stream(stream)), "MinimalFunctionLocal_gpu")


def petsc_vec_write(path, x, append=False):
    """Write a float64 host array as a PETSc binary Vec (natural ordering)."""
    import numpy as np
    a = np.ascontiguousarray(x, dtype=np.float64).ravel()
    _check(load().fishgpu_petsc_vec_write(str(path).encode(), int(append), a.ctypes.data, a.size),
           "fishgpu_petsc_vec_write")


def petsc_vec_read(path, index=0):
    """The index-th object of a PETSc binary file, which must be a Vec."""
    import numpy as np
    n = c_ll()
    _check(load().fishgpu_petsc_vec_read(str(path).encode(), index, None, 0, ctypes.byref(n)),
           "fishgpu_petsc_vec_read")
    a = np.empty(n.value)
    _check(load().fishgpu_petsc_vec_read(str(path).encode(), index, a.ctypes.data, a.size, ctypes.byref(n)),
           "fishgpu_petsc_vec_read")
    return a


def petsc_mat_write(path, csr, append=False):
    """Write a scipy CSR matrix as a PETSc binary AIJ Mat."""
    import numpy as np
    rp = np.ascontiguousarray(csr.indptr, dtype=np.int64)
    col = np.ascontiguousarray(csr.indices, dtype=np.int32)
    val = np.ascontiguousarray(csr.data, dtype=np.float64)
    M, N = csr.shape
    _check(load().fishgpu_petsc_mat_write_aij(str(path).encode(), int(append), M, N, rp.ctypes.data,
                                              col.ctypes.data, val.ctypes.data), "fishgpu_petsc_mat_write_aij")


def petsc_mat_read(path, index=0):
    """The index-th object of a PETSc binary file, which must be an AIJ Mat:
    returns (M, N, rowptr, col, val)."""
    import numpy as np
    M, N, nz = c_int(), c_int(), c_ll()
    p = str(path).encode()
    _check(load().fishgpu_petsc_mat_read_aij(p, index, ctypes.byref(M), ctypes.byref(N), ctypes.byref(nz), None,
                                             None, None), "fishgpu_petsc_mat_read_aij")
    rp = np.empty(M.value + 1, np.int64)
    col = np.empty(nz.value, np.int32)
    val = np.empty(nz.value)
    _check(load().fishgpu_petsc_mat_read_aij(p, index, ctypes.byref(M), ctypes.byref(N), ctypes.byref(nz),
                                             rp.ctypes.data, col.ctypes.data, val.ctypes.data),
           "fishgpu_petsc_mat_read_aij")
    return M.value, N.value, rp, col, val


def solve(opts, u=None):
    """Run the fish flow; returns (u, report).  u: CUDA float64 tensor (mz,my,mx)."""
    import torch
    if u is None:
        u = torch.empty(opts.shape, dtype=torch.float64, device="cuda")
    with Solver(opts) as s:
        rep = s.solve(u)
    return u, rep
