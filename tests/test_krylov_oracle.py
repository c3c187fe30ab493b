"""The oracle's GMRES(m) restatement against direct solves (CPU)."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from krylov_oracle import block_jacobi, gmres_left


def convection_diffusion(n, ns=1, seed=0):
    """Nonsymmetric, diagonally dominant block matrix on an n x n grid."""
    rng = np.random.default_rng(seed)
    N = n * n
    rows, cols, vals = [], [], []
    for K in range(N):
        i, j = divmod(K, n)
        nbrs = [(i + di) * n + (j + dj) for di, dj in ((1, 0), (-1, 0), (0, 1), (0, -1))
                if 0 <= i + di < n and 0 <= j + dj < n]
        for a in range(ns):
            for b in range(ns):
                rows.append(K * ns + a); cols.append(K * ns + b)
                vals.append(4.5 + rng.uniform() if a == b else 0.3 * rng.uniform())
            for M in nbrs:
                rows.append(K * ns + a); cols.append(M * ns + a)
                vals.append(-1.0 + 0.4 * (M - K > 0) * rng.uniform())
    return sp.csr_matrix((vals, (rows, cols)), shape=(N * ns, N * ns))


@pytest.mark.parametrize("m", [5, 30])
@pytest.mark.parametrize("ns", [1, 3])
def test_gmres_matches_direct_solve(m, ns):
    A = convection_diffusion(12, ns, seed=m + ns)
    b = np.random.default_rng(1).normal(size=A.shape[0])
    x, it = gmres_left(A, b, block_jacobi(A, ns), m=m, reltol=1e-12, maxiters=2000)
    xd = spla.spsolve(A.tocsc(), b)
    assert 0 < it < 2000
    assert np.max(np.abs(x - xd)) <= 1e-9 * np.max(np.abs(xd))


def test_gmres_residual_estimate_is_true_residual():
    # without restarts the least-squares residual is the preconditioned residual
    A = convection_diffusion(10, 1, seed=3)
    b = np.random.default_rng(2).normal(size=A.shape[0])
    minv = block_jacobi(A, 1)
    tol = 1e-6
    x, it = gmres_left(A, b, minv, m=32, reltol=tol, maxiters=32)
    true = np.linalg.norm(minv(b - A @ x))
    assert it < 32
    assert true <= 1.0001 * tol * np.linalg.norm(minv(b))


def test_gmres_finite_termination_and_zero_rhs():
    A = convection_diffusion(3, 1, seed=4)  # 9 unknowns
    b = np.arange(1.0, 10.0)
    x, it = gmres_left(A, b, lambda v: v, m=32, reltol=1e-14, maxiters=100)
    assert it <= 9
    assert np.allclose(A @ x, b, rtol=0, atol=1e-10)
    x0, it0 = gmres_left(A, np.zeros(9), lambda v: v, m=4)
    assert it0 == 0 and not x0.any()


def test_gmres_restart_needs_more_iterations():
    A = convection_diffusion(16, 1, seed=5)
    b = np.ones(A.shape[0])
    minv = block_jacobi(A, 1)
    _, it_full = gmres_left(A, b, minv, m=32, reltol=1e-10, maxiters=5000)
    _, it_short = gmres_left(A, b, minv, m=4, reltol=1e-10, maxiters=5000)
    assert it_short >= it_full
