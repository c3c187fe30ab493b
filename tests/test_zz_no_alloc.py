"""The allocation-free linear solve (vfvm_linsolve_csr_noalloc).

It exists for callers that cannot call cudaMalloc where they solve: their
device memory is owned by a framework's pool, allocation is forbidden in the
calling region, or they only have fixed pre-reserved buffers.  It must give the
same answer as the allocating entry point (vfvm_linsolve_csr) on the same
input, on repeated calls that share its fixed work array, and it must refuse
systems larger than that array with a clear status.

This file is collected last on purpose, so a failure here comes after every
other test has run; it also passes when run alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest
import scipy.sparse as sp

from gpu_cases import lin

pytestmark = pytest.mark.gpu
TOL = 1e-10  # agreement between the two entry points (both iterate to reltol 1e-12)


@pytest.fixture(scope="module")
def torch():
    return pytest.importorskip("torch")


def run(lib, fn, torch, A, b):
    A = sp.csr_matrix(A)
    A.sort_indices()
    rp = torch.from_numpy(A.indptr.astype(np.int32)).cuda()
    ci = torch.from_numpy(A.indices.astype(np.int32)).cuda()
    vv = torch.from_numpy(A.data.astype(np.float64)).cuda()
    bd = torch.from_numpy(np.ascontiguousarray(b, dtype=np.float64)).cuda()
    xd = torch.full_like(bd, np.nan)  # the solver must overwrite every entry
    it = ctypes.c_int32(0)
    res = ctypes.c_double(0)
    rc = getattr(lib, fn)(A.shape[0], A.nnz, rp.data_ptr(), ci.data_ptr(), vv.data_ptr(), bd.data_ptr(),
                          xd.data_ptr(), 1e-12, 0.0, 2000, ctypes.byref(it), ctypes.byref(res))
    return rc, xd.cpu().numpy(), it.value


def problem(oracle, vfvm, n, seed):
    g = vfvm.simplexgrid(lin(n), lin(n))
    osys = oracle.OracleSystem(g, "nlpoisson")
    u = np.random.default_rng(seed).uniform(0.0, 0.5, size=g.nnodes)
    osys.init_dirichlet(u)
    F, J = osys.assemble(u)
    return J, F


def test_noalloc_matches_allocating_solve_twice(vfvm, oracle, torch):
    lib = vfvm._lib.load()
    # two different systems in a row: the second call must not see the first one's leftovers
    for n, seed in ((48, 1), (31, 2)):
        J, F = problem(oracle, vfvm, n, seed)
        rc_ref, x_ref, it_ref = run(lib, "vfvm_linsolve_csr", torch, J, F)
        rc, x, it = run(lib, "vfvm_linsolve_csr_noalloc", torch, J, F)
        assert rc_ref == 0 and rc == 0
        assert np.all(np.isfinite(x))
        assert np.max(np.abs(x - x_ref)) <= TOL * np.max(np.abs(x_ref))
        assert it == it_ref


def test_noalloc_near_its_row_limit(vfvm, oracle, torch):
    """A 362 x 362 grid (131044 rows, just below the limit of 131072) exercises
    the fixed layout of the work array at nearly full size.  The matrix is an
    implicit Euler Jacobian with a short time step, so Jacobi BiCGStab
    converges quickly."""
    lib = vfvm._lib.load()
    g = vfvm.simplexgrid(lin(361), lin(361))
    assert vfvm._lib.NOALLOC_MAX_ROWS - 64 < g.nnodes <= vfvm._lib.NOALLOC_MAX_ROWS
    osys = oracle.OracleSystem(g, "porous")
    rng = np.random.default_rng(5)
    u = rng.uniform(0.2, 0.8, size=g.nnodes)
    F, J = osys.assemble(u, rng.uniform(0.2, 0.8, size=g.nnodes), 0.0, 1e-6)
    rc_ref, x_ref, it_ref = run(lib, "vfvm_linsolve_csr", torch, J, F)
    rc, x, it = run(lib, "vfvm_linsolve_csr_noalloc", torch, J, F)
    assert rc_ref == 0 and rc == 0
    assert np.all(np.isfinite(x))
    assert np.max(np.abs(x - x_ref)) <= TOL * np.max(np.abs(x_ref))
    assert it == it_ref
    # the solution solves the system
    assert np.max(np.abs(J @ x - F)) <= 1e-9 * np.max(np.abs(F))


def test_noalloc_rejects_oversized_system(vfvm, torch):
    lib = vfvm._lib.load()
    n = vfvm._lib.NOALLOC_MAX_ROWS + 1
    A = sp.identity(n, format="csr")
    rc, _, _ = run(lib, "vfvm_linsolve_csr_noalloc", torch, A, np.ones(n))
    assert rc == vfvm._lib.ERR_NOALLOC_LIMIT
