"""CPU oracle of the nonlinear clients of the Poisson call-backs (test
infrastructure only): the minimal-surface equation of c/ch7/minimal.c and the
Liouville-Bratu equation of c/ch7/solns/bratu2D.c (ctypes bindings of
oracle/minimal_oracle.c and oracle/bratu_oracle.c), plus a restatement of
PETSc's SNESNEWTONLS with the cubic backtracking line search and
SNESConvergedDefault, using exact sparse linear solves (scipy).

Newton steps here solve J Y = F exactly; the reference's runs solve them to
KSP rtol 1e-5, so intermediate residual norms agree to about that relative
size and converged quantities (errors, areas of converged iterates, iteration
counts) agree closely.
"""
import ctypes
import math

import numpy as np

import _oracle

TENT, CATENOID = 0, 1
REASONS = {2: "CONVERGED_FNORM_ABS", 3: "CONVERGED_FNORM_RELATIVE", 4: "CONVERGED_SNORM_RELATIVE",
           -5: "DIVERGED_MAX_IT", -6: "DIVERGED_LINE_SEARCH", -4: "DIVERGED_FNORM_NAN"}


class MsGrid(ctypes.Structure):
    _fields_ = [("mx", ctypes.c_int), ("my", ctypes.c_int), ("problem", ctypes.c_int), ("q", ctypes.c_double),
                ("catenoid_c", ctypes.c_double), ("tent_H", ctypes.c_double)]


class NkReport(ctypes.Structure):
    _fields_ = [("ngrids", ctypes.c_int), ("m", ctypes.c_int * 16), ("its", ctypes.c_int * 16),
                ("reason", ctypes.c_int * 16), ("ksp_its", ctypes.c_longlong), ("errinf", ctypes.c_double),
                ("fnorm_last", ctypes.c_double)]


_bound = False


def lib():
    global _bound
    L = _oracle.lib()
    if not _bound:
        P = ctypes.POINTER
        dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
        ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
        L.ms_g.argtypes = [P(MsGrid), ctypes.c_double, ctypes.c_double]
        L.ms_g.restype = ctypes.c_double
        L.ms_initial.argtypes = [P(MsGrid), dp]
        L.ms_exact.argtypes = [P(MsGrid), dp]
        L.ms_residual.argtypes = [P(MsGrid), dp, dp]
        L.ms_jv.argtypes = [P(MsGrid), dp, dp, dp]
        L.ms_jacobian_csr.argtypes = [P(MsGrid), dp, ip, ip, dp]
        L.ms_jacobian_csr.restype = ctypes.c_int
        L.ms_area.argtypes = [P(MsGrid), dp, ctypes.c_int, P(ctypes.c_double), P(ctypes.c_double),
                              P(ctypes.c_double)]
        L.ms_interpolate.argtypes = [P(MsGrid), dp, P(MsGrid), dp]
        L.ms_nk_solve.argtypes = [P(MsGrid), ctypes.c_int, ctypes.c_double, ctypes.c_double, dp, P(NkReport)]
        L.ms_nk_solve.restype = ctypes.c_int
        _bound = True
    return L


def grid(m, problem=CATENOID, q=-0.5, c=1.1, H=1.0):
    return MsGrid(m, m, problem, q, c, H)


def initial(g):
    u = np.empty(g.mx * g.my)
    lib().ms_initial(ctypes.byref(g), u)
    return u


def exact(g):
    u = np.empty(g.mx * g.my)
    lib().ms_exact(ctypes.byref(g), u)
    return u


def residual(g, u):
    F = np.empty_like(u)
    lib().ms_residual(ctypes.byref(g), np.ascontiguousarray(u), F)
    return F


def jv(g, u, v):
    out = np.empty_like(u)
    lib().ms_jv(ctypes.byref(g), np.ascontiguousarray(u), np.ascontiguousarray(v), out)
    return out


def jacobian(g, u):
    import scipy.sparse as sp
    n = g.mx * g.my
    rp = np.empty(n + 1, np.int32)
    col = np.empty(9 * n, np.int32)
    val = np.empty(9 * n)
    nz = lib().ms_jacobian_csr(ctypes.byref(g), np.ascontiguousarray(u), rp, col, val)
    return sp.csr_matrix((val[:nz], col[:nz], rp), shape=(n, n))


def area(g, u, degree=3):
    a, lo, hi = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    lib().ms_area(ctypes.byref(g), np.ascontiguousarray(u), degree, ctypes.byref(a), ctypes.byref(lo),
                  ctypes.byref(hi))
    return a.value, lo.value, hi.value


def interpolate(gc, uc, gf):
    uf = np.empty(gf.mx * gf.my)
    lib().ms_interpolate(ctypes.byref(gc), np.ascontiguousarray(uc), ctypes.byref(gf), uf)
    return uf


class LbGrid(ctypes.Structure):
    _fields_ = [("mx", ctypes.c_int), ("my", ctypes.c_int), ("lam", ctypes.c_double), ("exact", ctypes.c_int)]


_lb_bound = False


def _lb():
    global _lb_bound
    L = lib()
    if not _lb_bound:
        P = ctypes.POINTER
        dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
        ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
        L.lb_exact.argtypes = [P(LbGrid), dp]
        L.lb_residual.argtypes = [P(LbGrid), dp, dp]
        L.lb_jacobian_csr.argtypes = [P(LbGrid), dp, ip, ip, dp]
        L.lb_jacobian_csr.restype = ctypes.c_int
        _lb_bound = True
    return L


class Bratu:
    """The Bratu residual/Jacobian on an mx x my grid (bratu2D.c)."""

    def __init__(self, m, lam=1.0, exact=False):
        self.g = LbGrid(m, m, lam, int(exact))
        self.mx = self.my = m

    def residual(self, u):
        F = np.empty_like(u)
        _lb().lb_residual(ctypes.byref(self.g), np.ascontiguousarray(u), F)
        return F

    def jacobian(self, u):
        import scipy.sparse as sp
        n = self.mx * self.my
        rp = np.empty(n + 1, np.int32)
        col = np.empty(5 * n, np.int32)
        val = np.empty(5 * n)
        nz = _lb().lb_jacobian_csr(ctypes.byref(self.g), np.ascontiguousarray(u), rp, col, val)
        return sp.csr_matrix((val[:nz], col[:nz], rp), shape=(n, n))

    def exact(self):
        u = np.empty(self.mx * self.my)
        _lb().lb_exact(ctypes.byref(self.g), u)
        return u


class Minimal:
    def __init__(self, g):
        self.g = g

    def residual(self, u):
        return residual(self.g, u)

    def jacobian(self, u):
        return jacobian(self.g, u)


def line_search_bt(g, X, F, fnorm, Y, J, alpha=1e-4, maxstep=1e8, minlambda=1e-12, max_it=40):
    """Cubic backtracking (Dennis & Schnabel A6.3.1) on f = ||F||^2 / 2 along
    X - lambda Y, PETSc's SNESLINESEARCHBT defaults.  Returns
    (ok, X, F, fnorm, lambda, ynorm, nfuncs)."""
    ynorm = np.linalg.norm(Y)
    if ynorm > maxstep:
        Y = Y * (maxstep / ynorm)
        ynorm = maxstep
    initslope = float(F @ (J @ Y))
    if initslope > 0.0:
        initslope = -initslope
    if initslope == 0.0:
        initslope = -1.0
    res = g.residual if hasattr(g, "residual") else (lambda w: residual(g, w))
    lam = 1.0
    W = X - lam * Y
    G = res(W)
    gnorm = np.linalg.norm(G)
    nf = 1
    if 0.5 * gnorm * gnorm <= 0.5 * fnorm * fnorm + lam * alpha * initslope:
        return True, W, G, gnorm, lam, lam * ynorm, nf
    # quadratic
    lamtemp = -initslope / (gnorm * gnorm - fnorm * fnorm - 2.0 * lam * initslope)
    lamprev, gprev = lam, gnorm
    lam = 0.5 * lam if lamtemp > 0.5 * lam else (0.1 * lam if lamtemp <= 0.1 * lam else lamtemp)
    for _ in range(max_it):
        if lam < minlambda:
            return False, X, F, fnorm, 0.0, 0.0, nf
        W = X - lam * Y
        G = res(W)
        gnorm = np.linalg.norm(G)
        nf += 1
        if 0.5 * gnorm * gnorm <= 0.5 * fnorm * fnorm + lam * alpha * initslope:
            return True, W, G, gnorm, lam, lam * ynorm, nf
        t1 = 0.5 * (gnorm * gnorm - fnorm * fnorm) - lam * initslope
        t2 = 0.5 * (gprev * gprev - fnorm * fnorm) - lamprev * initslope
        a = (t1 / (lam * lam) - t2 / (lamprev * lamprev)) / (lam - lamprev)
        b = (-lamprev * t1 / (lam * lam) + lam * t2 / (lamprev * lamprev)) / (lam - lamprev)
        d = max(b * b - 3.0 * a * initslope, 0.0)
        lamtemp = -initslope / (2.0 * b) if a == 0.0 else (-b + math.sqrt(d)) / (3.0 * a)
        lamprev, gprev = lam, gnorm
        lam = 0.5 * lam if lamtemp > 0.5 * lam else (0.1 * lam if lamtemp <= 0.1 * lam else lamtemp)
    return False, X, F, fnorm, 0.0, 0.0, nf


def newton(g, u0, rtol=1e-8, atol=1e-50, stol=1e-8, max_it=50, monitor_degree=0):
    """PETSc SNESNEWTONLS + SNESConvergedDefault with exact linear solves.
    Returns a dict: u, its, reason, fnorms, areas (per iterate when
    monitor_degree > 0: (area, Dmin, Dmax))."""
    from scipy.sparse.linalg import spsolve
    model = g if hasattr(g, "residual") else Minimal(g)
    X = np.array(u0, dtype=np.float64)
    F = model.residual(X)
    fnorm = np.linalg.norm(F)
    fnorms = [fnorm]
    areas = [area(g, X, monitor_degree)] if monitor_degree else []  # minimal surface only
    ttol = rtol * fnorm
    reason = 0
    if math.isnan(fnorm):
        reason = -4
    elif fnorm < atol:
        reason = 2
    its = 0
    while reason == 0:
        J = model.jacobian(X)
        Y = spsolve(J.tocsc(), F)
        ok, X, F, fnorm, lam, ynorm, _ = line_search_bt(model, X, F, fnorm, Y, J)
        its += 1
        fnorms.append(fnorm)
        if monitor_degree:
            areas.append(area(g, X, monitor_degree))
        if not ok:
            reason = -6
            break
        xnorm = np.linalg.norm(X)
        if math.isnan(fnorm):
            reason = -4
        elif fnorm < atol:
            reason = 2
        elif fnorm <= ttol:
            reason = 3
        elif ynorm < stol * xnorm:
            reason = 4
        elif its >= max_it:
            reason = -5
    return {"u": X, "its": its, "reason": reason, "fnorms": fnorms, "areas": areas}


def solve(base=3, refine=0, grid_sequence=0, problem=CATENOID, q=-0.5, c=1.1, H=1.0, exact_init=False,
          monitor_degree=0, rtol=1e-8):
    """minimal.c's flow: the DMDA of base x base nodes refined `refine` times,
    then `grid_sequence` more grids, each solved from the interpolation of the
    previous solution.  Returns (levels, final_grid, u, errinf or None)."""
    m = base
    for _ in range(refine):
        m = 2 * m - 1
    levels = []
    g = grid(m, problem, q, c, H)
    u0 = exact(g) if exact_init else initial(g)
    for lev in range(grid_sequence + 1):
        r = newton(g, u0, rtol=rtol, monitor_degree=monitor_degree)
        r["m"] = g.mx
        levels.append(r)
        if lev < grid_sequence:
            gf = grid(2 * g.mx - 1, problem, q, c, H)
            u0 = interpolate(g, r["u"], gf)
            g = gf
    u = levels[-1]["u"]
    err = None
    if problem == CATENOID and q == -0.5:
        err = float(np.max(np.abs(u - exact(g))))
    return levels, g, u, err


def bratu_solve(base=3, refine=0, grid_sequence=0, lam=1.0, exact=False, rtol=1e-8):
    """bratu2D.c's Newton flow from u = 0 (bratu2D.c:133-135) with optional
    grid sequencing; returns (levels, model, u, errinf or None)."""
    m = base
    for _ in range(refine):
        m = 2 * m - 1
    levels = []
    model = Bratu(m, lam, exact)
    u0 = np.zeros(m * m)
    for lev in range(grid_sequence + 1):
        r = newton(model, u0, rtol=rtol)
        r["m"] = model.mx
        levels.append(r)
        if lev < grid_sequence:
            fine = Bratu(2 * model.mx - 1, lam, exact)
            u0 = interpolate(grid(model.mx), r["u"], grid(fine.mx))
            model = fine
    u = levels[-1]["u"]
    err = float(np.max(np.abs(u - model.exact()))) if exact else None
    return levels, model, u, err


def nk_solve(base=33, grid_sequence=5, rtol=1e-10, ksp_rtol=1e-5, problem=CATENOID, q=-0.5, c=1.1, H=1.0):
    """The GPU library's method on the CPU (oracle/ms_nk.c): Newton with the
    cubic line search, BiCGStab right-preconditioned with the Poisson V-cycle,
    grid sequencing; FP64, OpenMP.  Returns (u of the last grid, report)."""
    g = grid(base, problem, q, c, H)
    m = base
    for _ in range(grid_sequence):
        m = 2 * m - 1
    u = np.empty(m * m)
    rep = NkReport()
    rc = lib().ms_nk_solve(ctypes.byref(g), grid_sequence, rtol, ksp_rtol, u, ctypes.byref(rep))
    assert rc == 0, rc
    return u, rep
