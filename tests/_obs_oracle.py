"""CPU oracle of the obstacle problem of c/ch12/obstacle.c (test
infrastructure only): psi, the exact solution, Poisson2DFunctionLocal with
f = 0 and g = the exact solution on (-2,2)^2, and a restatement of PETSc's
reduced-space active-set Newton for variational inequalities
(SNESVINEWTONRSLS: project the iterate onto u >= psi; active set
u <= psi + 1e-8 with F > 0; solve the Jacobian restricted to the inactive set
exactly; projected step; residual norm over the inactive set;
SNESConvergedDefault), plus the report of obstacle.c:147-183.
"""
import math

import numpy as np

AFREE, A_COEF, B_COEF = 0.697965148223374, 0.680259411891719, 0.471519893402112
ZEROTOL = 1.0e-8


def psi(x, y):
    """obstacle.c:15-25"""
    r = np.sqrt(x * x + y * y)
    r0 = 0.9
    psi0 = math.sqrt(1.0 - r0 * r0)
    dpsi0 = -r0 / psi0
    return np.where(r <= r0, np.sqrt(np.maximum(1.0 - r * r, 0.0)), psi0 + dpsi0 * (r - r0))


def u_exact(x, y):
    """obstacle.c:39-48"""
    r = np.sqrt(x * x + y * y)
    return np.where(r <= AFREE, psi(x, y), -A_COEF * np.log(np.maximum(r, 1e-300)) + B_COEF)


def coords(m):
    h = 4.0 / (m - 1)
    x = -2.0 + h * np.arange(m)
    X, Y = np.meshgrid(x, x)
    return h, X, Y


def residual(m, u):
    """Poisson2DFunctionLocal (c/ch6/poissonfunctions.c:27-64), cx = cy = 1,
    f = 0, g = u_exact: boundary neighbours of interior rows take g."""
    h, X, Y = coords(m)
    U = u.reshape(m, m)
    g = u_exact(X, Y)
    scx = scy = 1.0
    sd = 2.0 * (scx + scy)
    b = np.zeros((m, m), bool)
    b[0, :] = b[-1, :] = b[:, 0] = b[:, -1] = True
    V = np.where(b, g, U)
    F = np.empty_like(U)
    F[1:-1, 1:-1] = sd * U[1:-1, 1:-1] - scx * (V[1:-1, :-2] + V[1:-1, 2:]) - scy * (V[:-2, 1:-1] + V[2:, 1:-1])
    F[b] = sd * (U[b] - g[b])
    return F.ravel()


def jacobian(m):
    import scipy.sparse as sp
    rows, cols, vals = [], [], []
    for j in range(m):
        for i in range(m):
            k = j * m + i
            rows.append(k)
            cols.append(k)
            vals.append(4.0)
            if i in (0, m - 1) or j in (0, m - 1):
                continue
            for di, dj in ((1, 0), (-1, 0), (0, 1), (0, -1)):
                a, b = i + di, j + dj
                if a in (0, m - 1) or b in (0, m - 1):
                    continue
                rows.append(k)
                cols.append(b * m + a)
                vals.append(-1.0)
    return sp.csr_matrix((vals, (rows, cols)), shape=(m * m, m * m))


def active(m, u, F):
    h, X, Y = coords(m)
    return (u <= psi(X, Y).ravel() + ZEROTOL) & (F > 0.0)


def solve(m, u0=None, rtol=1e-8, atol=1e-50, stol=1e-8, max_it=50):
    import scipy.sparse.linalg as sla
    h, X, Y = coords(m)
    lo = psi(X, Y).ravel()
    u = np.maximum(np.zeros(m * m) if u0 is None else np.array(u0, float), lo)
    J = jacobian(m)
    F = residual(m, u)
    fnorm = np.linalg.norm(F[~active(m, u, F)])
    fnorms = [fnorm]
    ttol = rtol * fnorm
    its, reason = 0, 0
    while not reason:
        I = ~active(m, u, F)
        Y = np.zeros_like(u)
        Y[I] = sla.spsolve(J[I][:, I].tocsc(), F[I])
        W = np.maximum(u - Y, lo)
        G = residual(m, W)
        gnorm = np.linalg.norm(G[~active(m, W, G)])
        snorm = np.linalg.norm(Y)
        u, F, fnorm = W, G, gnorm
        its += 1
        fnorms.append(fnorm)
        if fnorm < atol:
            reason = 2
        elif fnorm <= ttol:
            reason = 3
        elif snorm < stol * np.linalg.norm(u):
            reason = 4
        elif its >= max_it:
            reason = -5
    return {"u": u, "its": its, "reason": reason, "fnorms": fnorms, "F": F}


def interpolate(uc, mc):
    mf = 2 * mc - 1
    U = uc.reshape(mc, mc)
    Fi = np.zeros((mf, mf))
    Fi[::2, ::2] = U
    Fi[1::2, ::2] = 0.5 * (U[:-1] + U[1:])
    Fi[::2, 1::2] = 0.5 * (U[:, :-1] + U[:, 1:])
    Fi[1::2, 1::2] = 0.25 * (U[:-1, :-1] + U[1:, :-1] + U[:-1, 1:] + U[1:, 1:])
    return Fi.ravel()


def run(base=3, refine=0, grid_sequence=0, rtol=1e-8):
    m = base
    for _ in range(refine):
        m = 2 * m - 1
    levels, u = [], None
    for lev in range(grid_sequence + 1):
        r = solve(m, u, rtol=rtol)
        r["m"] = m
        levels.append(r)
        if lev < grid_sequence:
            u = interpolate(r["u"], m)
            m = 2 * m - 1
    return levels


def report(m, u, F):
    """errors: av |u-uexact|, |u-uexact|_inf, active area error (obstacle.c:147-183)"""
    h, X, Y = coords(m)
    e = u - u_exact(X, Y).ravel()
    nact = int(active(m, u, F).sum())
    exact = math.pi * AFREE * AFREE
    return np.abs(e).sum() / (m * m), np.abs(e).max(), abs(h * h * nact - exact) / exact, nact
