"""GMRES(m) on the persistent engine: Krylov iteration counts against the
oracle's GMRES restatement (FP64, block Jacobi), and Newton solutions with
every preconditioner against the oracle's FP64 solution (<= 1e-8 relative)."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

from gpu_cases import lin
from krylov_oracle import block_jacobi, gmres_left

pytestmark = pytest.mark.gpu
SOL_TOL = 1e-8


def rel_err(a, b):
    a = np.asarray(a).ravel(order="F")
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def kappa_case(vfvm, n, seed, f):
    g = vfvm.simplexgrid(lin(n), lin(n))
    kappa = np.exp(np.random.default_rng(seed).normal(size=g.nnodes))
    return g, kappa, vfvm.Physics("kappa_exp", [f], kappa)


@pytest.mark.parametrize("restart", [4, 10, 32])
def test_gmres_iterations_match_oracle(vfvm, oracle, restart):
    # one linear solve (is_linear): the device's Arnoldi step count equals the
    # oracle restatement's on the same Jacobian, restarts included
    g, kappa, phys = kappa_case(vfvm, 24, 11, 0.7)
    sys = vfvm.System(g, phys, is_linear=True)
    control = vfvm.SolverControl(method_linear="gmres", gmres_restart=restart, precon_linear="jacobi",
                                 precision="fp64", reltol_linear=1e-8, maxiters_linear=3000)
    U = vfvm.solve(sys, inival=0.0, control=control)
    nlin = vfvm.solve.last_history.nlin
    osys = oracle.OracleSystem(g, "kappa_exp", [0.7], nodedata=kappa)
    u0 = osys.init_dirichlet(np.zeros(osys.n))
    F, J = osys.assemble(u0)
    x, it = gmres_left(J, F, block_jacobi(J, 1), m=restart, reltol=1e-8, maxiters=3000)
    assert it > restart  # the case exercises restarts
    assert abs(nlin - it) <= 1
    assert rel_err(U, u0 - x) <= 1e-6
    assert rel_err(U, u0 - spla.spsolve(J.tocsc(), F)) <= 1e-6


@pytest.mark.parametrize("precon", ["jacobi", "ilu0", "block_ilu0"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gmres_newton_vs_oracle(vfvm, oracle, precon, precision):
    g = vfvm.simplexgrid(lin(32), lin(32))
    sys = vfvm.System(g, vfvm.Physics("nlpoisson"))
    control = vfvm.SolverControl(method_linear="gmres", gmres_restart=20, precon_linear=precon, precision=precision,
                                 maxiters_linear=600)
    U = vfvm.solve(sys, inival=0.0, control=control)
    assert vfvm.solve.last_history.nlin > 0
    osys = oracle.OracleSystem(g, "nlpoisson", [])
    u, _ = oracle.solve_step(osys, np.zeros(osys.n), oracle.Control())
    assert rel_err(U, u) <= SOL_TOL


@pytest.mark.parametrize("precon", ["ilu0", "block_ilu0"])
def test_gmres_coarse_stage_vs_oracle(vfvm, oracle, precon):
    g, kappa, phys = kappa_case(vfvm, 40, 6, -0.4)
    sys = vfvm.System(g, phys)
    base = dict(method_linear="gmres", gmres_restart=30, precon_linear=precon, maxiters_linear=2000)
    vfvm.solve(sys, inival=0.0, control=vfvm.SolverControl(**base))
    lin_plain = vfvm.solve.last_history.nlin
    U = vfvm.solve(sys, inival=0.0, control=vfvm.SolverControl(coarse=100, **base))
    lin_coarse = vfvm.solve.last_history.nlin
    osys = oracle.OracleSystem(g, "kappa_exp", [-0.4], nodedata=kappa)
    u, _ = oracle.solve_step(osys, np.zeros(osys.n), oracle.Control())
    assert rel_err(U, u) <= SOL_TOL
    assert lin_coarse < 0.7 * lin_plain


def test_gmres_fixed_steps_vs_oracle(vfvm, oracle):
    # implicit Euler steps inside one persistent launch, GMRES for every Newton step
    g = vfvm.simplexgrid(lin(32), lin(32))
    x, y = g.coord
    u0 = 1e-3 + np.exp(-((x - 0.5) ** 2 + (y - 0.5) ** 2) / 0.1 ** 2)
    sys = vfvm.System(g, vfvm.Physics("porous"))
    control = vfvm.fixed_timesteps(vfvm.SolverControl(method_linear="gmres", gmres_restart=16), 1e-3)
    tsol = vfvm.solve(sys, inival=u0.reshape(1, -1), times=[0.0, 0.005], control=control)
    osys = oracle.OracleSystem(g, "porous")
    _, osols, _ = oracle.solve_transient(osys, u0, [0.0, 0.005], oracle.fixed_timesteps(oracle.Control(), 1e-3))
    assert rel_err(tsol.u[-1], osols[-1]) <= SOL_TOL


def test_gmres_rejected_outside_persistent_engine(vfvm):
    sys = vfvm.System(vfvm.simplexgrid(lin(8), lin(8)), vfvm.Physics("nlpoisson"))
    with pytest.raises(ValueError):
        vfvm.solve(sys, inival=0.0, control=vfvm.SolverControl(method_linear="gmres", engine="graph"))
    for restart in (0, 33):
        with pytest.raises(ValueError):
            vfvm.solve(sys, inival=0.0, control=vfvm.SolverControl(method_linear="gmres", gmres_restart=restart))
    # a system above the automatic persistent-engine size still runs GMRES persistently
    big = vfvm.System(vfvm.simplexgrid(lin(160), lin(160)), vfvm.Physics("nlpoisson"))
    U = vfvm.solve(big, inival=0.0, control=vfvm.SolverControl(method_linear="gmres", maxiters_linear=800))
    assert np.isfinite(U).all() and U.max() > 0
