"""Device CSR linear solve (the reference's method_linear plug point) against a
sparse direct solve, through the C ABI."""
import ctypes

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from gpu_cases import lin

pytestmark = pytest.mark.gpu


def device_csr(torch, A):
    A = sp.csr_matrix(A)
    A.sort_indices()
    rp = torch.from_numpy(A.indptr.astype(np.int32)).cuda()
    ci = torch.from_numpy(A.indices.astype(np.int32)).cuda()
    vv = torch.from_numpy(A.data.astype(np.float64)).cuda()
    return A, rp, ci, vv


def solve(vfvm, torch, A, b, reltol=1e-12, maxiters=2000):
    lib = vfvm._lib.load()
    A, rp, ci, vv = device_csr(torch, A)
    bd = torch.from_numpy(np.ascontiguousarray(b)).cuda()
    xd = torch.zeros_like(bd)
    it = ctypes.c_int32(0)
    res = ctypes.c_double(0)
    rc = lib.vfvm_linsolve_csr(A.shape[0], A.nnz, rp.data_ptr(), ci.data_ptr(), vv.data_ptr(), bd.data_ptr(),
                               xd.data_ptr(), reltol, 0.0, maxiters, ctypes.byref(it), ctypes.byref(res))
    return rc, xd.cpu().numpy(), it.value


@pytest.fixture(scope="module")
def torch():
    return pytest.importorskip("torch")


def test_linsolve_random_diag_dominant(vfvm, torch):
    rng = np.random.default_rng(0)
    n = 5000
    R = sp.random(n, n, density=5.0 / n, random_state=1, format="csr")
    A = R + sp.diags(np.abs(R).sum(axis=1).A1 + 1.0)
    b = rng.normal(size=n)
    rc, x, it = solve(vfvm, torch, A, b)
    assert rc == 0 and it > 0
    xs = spla.spsolve(A.tocsc(), b)
    assert np.max(np.abs(x - xs)) <= 1e-8 * np.max(np.abs(xs))


def test_linsolve_jacobian_with_penalty_rows(vfvm, torch, oracle):
    # a Newton Jacobian of the nonlinear Poisson workload: 1e30 penalty diagonal on boundary rows
    g = vfvm.simplexgrid(lin(40), lin(40))
    osys = oracle.OracleSystem(g, "nlpoisson")
    u = np.random.default_rng(2).uniform(0.0, 0.5, size=g.nnodes)
    osys.init_dirichlet(u)
    F, J = osys.assemble(u)
    rc, x, it = solve(vfvm, torch, J, F)
    assert rc == 0
    xs = spla.splu(J.tocsc()).solve(F)
    assert np.max(np.abs(x - xs)) <= 1e-8 * np.max(np.abs(xs))


def test_linsolve_rejects_bad_structure(vfvm, torch):
    A = sp.csr_matrix(sp.eye(100) * 2.0)
    A.indices[5] = 1000  # column outside [0, n)
    rc, _, _ = solve(vfvm, torch, A, np.ones(100))
    assert rc == vfvm._lib.ERR_INPUT
