"""ctypes bindings of the CPU oracle (oracle/_build/liboracle.so).

The oracle is the checker: only tests, __graft_entry__.smoke() and bench.py's
CPU-baseline leg use it.
"""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
LIB = os.path.join(ORACLE_DIR, "_build", "liboracle.so")
EXE = os.path.join(ORACLE_DIR, "_build", "fish_oracle")

MANUPOLY, MANUEXP, ZERO, USER = 0, 1, 2, 3
PC_NONE, PC_JACOBI, PC_MG, PC_ILU = 0, 1, 2, 3

c_int, c_double, c_void_p = ctypes.c_int, ctypes.c_double, ctypes.c_void_p


class Grid(ctypes.Structure):
    _fields_ = [("dim", c_int), ("mx", c_int), ("my", c_int), ("mz", c_int),
                ("Lx", c_double), ("Ly", c_double), ("Lz", c_double),
                ("cx", c_double), ("cy", c_double), ("cz", c_double),
                ("problem", c_int), ("f_user", c_void_p), ("g_user", c_void_p)]


class Opts(ctypes.Structure):
    _fields_ = [("grid", Grid), ("initial_type", c_int), ("initial_gonboundary", c_int),
                ("rtol", c_double), ("atol", c_double), ("dtol", c_double),
                ("max_it", c_int), ("norm_type", c_int), ("pc_type", c_int), ("mg_levels", c_int),
                ("mg_cycles", c_int), ("smooth_type", c_int), ("smooth_its", c_int),
                ("esteig", c_double * 4), ("richardson_scale", c_double),
                ("seed", ctypes.c_ulonglong)]


class Report(ctypes.Structure):
    _fields_ = [("its", c_int), ("reason", c_int), ("nhist", c_int),
                ("hist", ctypes.POINTER(c_double)), ("fnorm0", c_double), ("fnorm1", c_double),
                ("errinf", c_double), ("err2h", c_double)]


_lib = None


def build():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        P = ctypes.POINTER
        dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
        L.or_residual.argtypes = [P(Grid), dp, dp]
        L.or_apply.argtypes = [P(Grid), dp, dp]
        L.or_exact_fill.argtypes = [P(Grid), dp]
        L.or_initial_state.argtypes = [P(Grid), c_int, c_int, ctypes.c_ulonglong, dp]
        L.or_errnorms.argtypes = [P(Grid), dp, P(c_double), P(c_double)]
        L.or_dot.argtypes = [P(Grid), dp, dp]
        L.or_dot.restype = c_double
        L.or_restrict.argtypes = [P(Grid), P(Grid), dp, dp]
        L.or_prolong_add.argtypes = [P(Grid), P(Grid), dp, dp]
        L.or_exact_solve.argtypes = [P(Grid), dp, dp]
        L.or_ksp_solve.argtypes = [P(Opts), dp, dp, P(Report)]
        L.or_fish_solve.argtypes = [P(Opts), dp, P(Report)]
        L.or_opts_default.argtypes = [P(Opts)]
        L.or_opts_parse.argtypes = [P(Opts), c_int, P(ctypes.c_char_p), P(c_int)]
        L.or_num_threads.restype = c_int
        _lib = L
    return _lib


def grid(dim, mx, my=1, mz=1, problem=MANUPOLY, c=(1.0, 1.0, 1.0), L=(1.0, 1.0, 1.0)):
    g = Grid()
    g.dim, g.mx = dim, mx
    g.my = my if dim >= 2 else 1
    g.mz = mz if dim >= 3 else 1
    g.Lx, g.Ly, g.Lz = L
    g.cx, g.cy, g.cz = c
    g.problem = problem
    return g


def shape(g):
    return (g.mz, g.my, g.mx)


def residual(g, u):
    F = np.empty_like(u)
    lib().or_residual(ctypes.byref(g), u, F)
    return F


def apply(g, p):
    q = np.empty_like(p)
    lib().or_apply(ctypes.byref(g), p, q)
    return q


def exact(g):
    u = np.empty(shape(g))
    lib().or_exact_fill(ctypes.byref(g), u)
    return u


def initial(g, itype, gbdry, seed=0):
    u = np.empty(shape(g))
    lib().or_initial_state(ctypes.byref(g), itype, int(gbdry), seed, u)
    return u


def errnorms(g, u):
    a, b = c_double(), c_double()
    lib().or_errnorms(ctypes.byref(g), np.ascontiguousarray(u), ctypes.byref(a), ctypes.byref(b))
    return a.value, b.value


def exact_solve(g, b):
    x = np.empty_like(b)
    rc = lib().or_exact_solve(ctypes.byref(g), np.ascontiguousarray(b), x)
    assert rc == 0
    return x


def options(argv):
    """or_opts from fish's flags (the oracle's own parser)."""
    if isinstance(argv, str):
        argv = argv.split()
    o = Opts()
    lib().or_opts_default(ctypes.byref(o))
    arr = (ctypes.c_char_p * max(1, len(argv)))(*[a.encode() for a in argv])
    rc = lib().or_opts_parse(ctypes.byref(o), len(argv), arr, None)
    if rc:
        raise ValueError("oracle option parse failed: %d" % rc)
    return o


def fish_solve(o):
    """Returns (u, report dict) of the whole fish flow."""
    g = o.grid
    u = np.empty(shape(g))
    hist = (c_double * (o.max_it + 2))()
    rep = Report()
    rep.hist = hist
    rc = lib().or_fish_solve(ctypes.byref(o), u, ctypes.byref(rep))
    assert rc == 0, rc
    return u, {"its": rep.its, "reason": rep.reason, "hist": [hist[i] for i in range(rep.nhist)],
               "fnorm0": rep.fnorm0, "fnorm1": rep.fnorm1, "errinf": rep.errinf, "err2h": rep.err2h}


def run_main(argv):
    """The oracle's fish-compatible command line; returns stdout."""
    if not os.path.exists(EXE):
        build()
    if isinstance(argv, str):
        argv = argv.split()
    p = subprocess.run([EXE] + list(argv), stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                       env=dict(os.environ, OMP_NUM_THREADS="1"))
    assert p.returncode == 0, p.stderr
    return p.stdout


def weights(g):
    """Stencil weights of the oracle's residual (poissonfunctions.c:35-40 in 2D,
    :76-82 in 3D): off-diagonal sc per dimension and the diagonal 2 * sum(sc)."""
    h = [g.Lx / (g.mx - 1), g.Ly / (g.my - 1) if g.dim >= 2 else 1.0, g.Lz / (g.mz - 1) if g.dim >= 3 else 1.0]
    c = [g.cx, g.cy, g.cz]
    if g.dim == 2:
        sc = [c[0] * h[1] / h[0], c[1] * h[0] / h[1]]
    elif g.dim == 3:
        vol = h[0] * h[1] * h[2]
        sc = [c[d] * vol / (h[d] * h[d]) for d in range(3)]
    else:
        raise ValueError("weights: 2D and 3D grids only")
    return sc, 2.0 * sum(sc)


def exact_solve_dst(g, b):
    """The exact solve of or_exact_solve (sine-transform diagonalisation of the
    Jacobian: boundary rows x = b / scdiag, interior x = S Lambda^-1 S b), with
    scipy's orthonormal DST-I for the transforms instead of dense sine
    matrices, so that grids of 513^3 nodes solve in seconds.  2D and 3D."""
    from scipy import fft
    sc, scdiag = weights(g)
    x = b / scdiag
    inner = (slice(1, -1), slice(1, -1), slice(1, -1)) if g.dim == 3 else (slice(None), slice(1, -1), slice(1, -1))
    axes = (0, 1, 2) if g.dim == 3 else (1, 2)
    a = fft.dstn(b[inner], type=1, norm="ortho", axes=axes, workers=-1)
    lam = 0.0
    for d in range(g.dim):  # axis of dimension d: x is the last axis
        n = b.shape[2 - d] - 2
        ld = sc[d] * (2.0 - 2.0 * np.cos(np.pi * np.arange(1, n + 1) / (n + 1)))
        shp = [1, 1, 1]
        shp[2 - d] = n
        lam = lam + ld.reshape(shp)
    a /= lam
    x[inner] = fft.dstn(a, type=1, norm="ortho", axes=axes, workers=-1, overwrite_x=True)
    return x
