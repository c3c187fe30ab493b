"""CPU restatement of the device GMRES(m) -- test infrastructure only: the
product never imports this module; tests use it as the checker.

Restarted GMRES with left preconditioning, the Krylov method behind
LinearSolve.jl's ``KrylovJL_GMRES`` (Krylov.jl ``gmres``).  LinearSolve is a
dependency of the reference (Project.toml:72, compat "3.52.0, 4, 5") that is
not vendored; the method is the published algorithm of Saad & Schultz (1986):
Arnoldi on M^-1 A, Hessenberg columns reduced by Givens rotations, restart
after m steps from the true residual.  The reference selects it with an ILU(0)
preconditioner in examples/DevEx004_EquationBlock3D.jl:187 and
examples/DevEx005_Mixture.jl:290.

This restatement follows the device solver step for step so that FP64 Krylov
iteration counts agree up to rounding: block classical Gram-Schmidt in chunks
of 8 basis vectors with one re-orthogonalisation pass, and the stopping test
||M^-1 (b - A x)|| <= max(abstol, reltol ||M^-1 b||) on the least-squares
residual |g_{k+1}|.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp


def block_jacobi(J: sp.spmatrix, ns: int):
    """x -> D^-1 x with D the ns x ns diagonal blocks of J (dof order K*ns+i)."""
    n = J.shape[0]
    N = n // ns
    Jc = sp.csr_matrix(J)
    D = np.zeros((N, ns, ns))
    for i in range(ns):
        for j in range(ns):
            D[:, i, j] = Jc[np.arange(N) * ns + i, np.arange(N) * ns + j].A1
    Dinv = np.linalg.inv(D)
    return lambda x: np.einsum("kij,kj->ki", Dinv, x.reshape(N, ns)).ravel()


def gmres_left(A, b, minv, m: int = 30, reltol: float = 1e-4, abstol: float = 0.0, maxiters: int = 100,
               chunk: int = 8):
    """Solve M^-1 A x = M^-1 b from x = 0; returns (x, Arnoldi steps)."""
    n = len(b)
    zb = minv(b)
    x = np.zeros(n)
    beta = float(np.linalg.norm(zb))
    tol = max(abstol, reltol * beta)
    it = 0
    if not beta > tol or maxiters <= 0:
        return x, 0
    r = zb
    while True:
        V = np.zeros((m + 1, n))
        V[0] = r / beta
        R = np.zeros((m, m))
        g = np.zeros(m + 1)
        g[0] = beta
        cs = np.zeros(m)
        sn = np.zeros(m)
        k = 0
        stop = False
        while k < m:
            w = minv(A @ V[k])
            h = np.zeros(k + 2)
            for _ in range(2):
                for i0 in range(0, k + 1, chunk):
                    blk = V[i0:min(i0 + chunk, k + 1)]
                    c = blk @ w
                    w = w - c @ blk
                    h[i0:i0 + len(c)] += c
            hn = float(np.linalg.norm(w))
            V[k + 1] = w / hn if hn > 0 else w
            for i in range(k):
                t = cs[i] * h[i] + sn[i] * h[i + 1]
                h[i + 1] = -sn[i] * h[i] + cs[i] * h[i + 1]
                h[i] = t
            rr = float(np.hypot(h[k], hn))
            cs[k], sn[k] = (h[k] / rr, hn / rr) if rr > 0 else (1.0, 0.0)
            h[k] = rr
            g[k + 1] = -sn[k] * g[k]
            g[k] = cs[k] * g[k]
            R[:k + 1, k] = h[:k + 1]
            res = abs(g[k + 1])
            k += 1
            it += 1
            if not res > tol or not hn > 0 or it >= maxiters:
                stop = True
                break
        y = np.zeros(k)
        for i in range(k - 1, -1, -1):
            s = g[i] - R[i, i + 1:k] @ y[i + 1:k]
            y[i] = s / R[i, i] if R[i, i] != 0 else 0.0
        x = x + y @ V[:k]
        if stop:
            break
        r = zb - minv(A @ x)
        beta = float(np.linalg.norm(r))
        if not beta > tol:
            break
    return x, it
