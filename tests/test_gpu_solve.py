"""GPU Newton solves through the product API: the reference's golden values, and
the benchmark workloads (small instances) against the oracle's FP64 solution
(<= 1e-8 relative, the solution-parity bar)."""
import json
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN
from gpu_cases import BIPOLAR, lin

pytestmark = pytest.mark.gpu
RTOL = math.sqrt(np.finfo(float).eps)
SOL_TOL = 1e-8


@pytest.fixture(scope="module")
def testvals():
    with open(os.path.join(GOLDEN, "reference_testvals.json")) as f:
        return json.load(f)


def test_example105(vfvm, testvals):
    g = vfvm.simplexgrid(lin(10))
    sys = vfvm.System(g, vfvm.Physics("ex105", [1e-3]))
    vfvm.boundary_dirichlet(sys, 1, 1, 0.0)
    vfvm.boundary_dirichlet(sys, 1, 2, 1.0)
    U = vfvm.solve(sys, inival=vfvm.unknowns(sys, inival=0.5))
    assert U.sum() == pytest.approx(testvals["Example105_NonlinearPoisson1D"]["value"], rel=RTOL)


def barenblatt(x, t, m):
    tx = t ** (-1.0 / (m + 1.0))
    xx = (x * tx) ** 2
    xx = max(1 - xx * (m - 1) / (2.0 * m * (m + 1)), 0.0)
    return tx * xx ** (1.0 / (m - 1.0))


@pytest.mark.parametrize("step_control", ["device", "host"])
def test_example106_transient(vfvm, testvals, step_control):
    X = np.array([(i - 10) / 10 for i in range(21)])
    sys = vfvm.System(vfvm.simplexgrid(X), vfvm.Physics("ex106", [2.0]))
    inival = vfvm.unknowns(sys)
    inival[0, :] = [barenblatt(x, 0.001, 2.0) for x in X]
    control = vfvm.SolverControl(step_control=step_control)
    control.Δt_min = control.Δt_max = control.Δt = 1e-4
    control.Δu_opt = 1.0
    tsol = vfvm.solve(sys, inival=inival, times=[0.001, 0.01], control=control)
    assert tsol.u[-1].sum() == pytest.approx(testvals["Example106_NonlinearDiffusion1D"]["value"], rel=RTOL)
    assert len(tsol.t) == 91 and tsol.history.nsteps == 90
    if step_control == "device":
        # the 90 steps ran inside one graph launch: the call synchronised with
        # the host three times in all (set-up, end of the loop, stored solutions)
        assert vfvm.solve.last_host_syncs == 3


def test_example110_two_species(vfvm, testvals):
    g = vfvm.simplexgrid(lin(100))
    sys = vfvm.System(g, vfvm.Physics("ex110", [1.0, 1.0]), species=[1, 2])
    for ispec, (v1, v2) in enumerate([(1.0, 0.0), (1.0, 0.0)], start=1):
        vfvm.boundary_dirichlet(sys, ispec, 1, v1)
        vfvm.boundary_dirichlet(sys, ispec, 2, v2)
    U = vfvm.unknowns(sys, inival=0.0)
    control = vfvm.SolverControl(damp_initial=0.1)
    for xeps in [1.0, 0.5, 0.25, 0.1, 0.05, 0.025, 0.01]:
        sys.physics.data = (xeps, xeps)
        U = vfvm.solve(sys, inival=U, control=control)
    assert U.ravel(order="F")[4] == pytest.approx(testvals["Example110_ReactionDiffusion1D_TwoSpecies"]["value"], rel=RTOL)


@pytest.mark.parametrize("step_control", ["device", "host"])
def test_example160_bernoulli_sedan(vfvm, testvals, step_control):
    sys = vfvm.System(vfvm.simplexgrid(lin(20)), vfvm.Physics("ex160", [1e-3, -1.0, 5.0]), species=[1, 2])
    inival = vfvm.unknowns(sys)
    inival[0, :] = 0.0
    inival[1, :] = 0.5
    control = vfvm.SolverControl(Δt_min=1e-5, Δt=1e-5, Δt_grow=1.1, Δt_max=0.1, Δu_opt=0.1, damp_initial=0.5,
                                 step_control=step_control)
    tsol = vfvm.solve(sys, inival=inival, times=[0.0, 10.0], control=control)
    assert tsol.u[-1].sum() == pytest.approx(testvals["Example160_UnipolarDriftDiffusion1D"]["value"], rel=1e-5)
    if step_control == "device":
        # adaptive steps (accepted, rejected and grown on the device), one graph launch
        assert tsol.history.nsteps > 50 and vfvm.solve.last_host_syncs == 3


def test_device_step_control_matches_host(vfvm):
    """The device controller takes the host controller's decisions: the same
    accepted times and solutions that agree to the solution-parity bar, with
    rejected steps (a du_opt that forces retries) and several output intervals."""
    g = vfvm.simplexgrid(lin(12), lin(12))
    x, y = g.coord
    u0 = 1e-3 + np.exp(-((x - 0.5) ** 2 + (y - 0.5) ** 2) / 0.1 ** 2)
    out = {}
    for mode in ("host", "device"):
        sys = vfvm.System(g, vfvm.Physics("porous"))
        control = vfvm.SolverControl(step_control=mode, engine="graph", Δt=2e-3, Δt_min=1e-5, Δt_max=5e-3,
                                     Δu_opt=0.05, Δt_grow=1.5, maxiters_linear=400, reltol_linear=1e-8)
        out[mode] = vfvm.solve(sys, inival=u0.reshape(1, -1), times=[0.0, 0.004, 0.01, 0.02], control=control)
    h, d = out["host"], out["device"]
    assert len(h.t) == len(d.t) > 8
    np.testing.assert_allclose(d.t, h.t, rtol=1e-12, atol=1e-15)
    for uh, ud in zip(h.u, d.u):
        assert np.max(np.abs(ud - uh)) <= 1e-8 * np.max(np.abs(uh))
    assert d.history.nsteps == h.history.nsteps


def test_example207_2d_timesteps(vfvm, testvals):
    sys = vfvm.System(vfvm.simplexgrid(lin(10), lin(10)), vfvm.Physics("ex207", [1e-2]))
    vfvm.boundary_dirichlet(sys, 1, 2, 0.1)
    vfvm.boundary_dirichlet(sys, 1, 4, 0.1)
    inival = vfvm.unknowns(sys, inival=0.5)
    control = vfvm.SolverControl(reltol_linear=1e-5)
    t = 0.0
    while t < 1.0:
        t = t + 0.01
        U = vfvm.solve(sys, inival=inival, control=control, tstep=0.01)
        inival = U
    assert U.ravel(order="F")[14] == pytest.approx(testvals["Example207_NonlinearPoisson2D"]["value"], rel=RTOL)


def test_example301_3d(vfvm, testvals):
    sys = vfvm.System(vfvm.simplexgrid(lin(5), lin(5), lin(5)), vfvm.Physics("ex301"))
    vfvm.boundary_dirichlet(sys, 1, 5, 0.0)
    vfvm.boundary_dirichlet(sys, 1, 6, 0.0)
    U = vfvm.solve(sys)
    assert U.ravel(order="F")[42] == pytest.approx(testvals["Example301_Laplace3D"]["value"], rel=RTOL)


def test_example440_parallel_states(vfvm, testvals):
    sys = vfvm.System(vfvm.simplexgrid(np.array([i / 320 for i in range(321)])), vfvm.Physics("ex440", [0.0]))
    total = 0.0
    for i in range(100):
        U = vfvm.solve(sys, inival=0.1, data=(i * 10.0 / 99.0,), abstol=1e-15, reltol=1e-20,
                       reltol_linear=1e-12, maxiters_linear=1000)
        total += float(vfvm.integrate(sys, U)[0])
    assert total == pytest.approx(testvals["Example440_ParallelState"]["value"], rel=RTOL)


# --- benchmark workloads (reduced sizes) against the oracle -----------------------------------

def oracle_solution(oracle, g, kind, params, nodedata=None, inival=None, tstep=math.inf, embed=0.0, control=None):
    osys = oracle.OracleSystem(g, kind, params, nodedata=nodedata)
    u0 = np.zeros(osys.n) if inival is None else np.asarray(inival, dtype=float).ravel(order="F")
    u, _ = oracle.solve_step(osys, u0, control or oracle.Control(), 0.0, tstep, embed)
    return u


def rel_err(a, b):
    a = np.asarray(a).ravel(order="F")
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("engine", ["persistent", "graph"])
@pytest.mark.parametrize("precon", ["ilu0", "jacobi", "block_ilu0"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nlpoisson_vs_oracle(vfvm, oracle, precon, precision, engine):
    g = vfvm.simplexgrid(lin(32), lin(32))
    sys = vfvm.System(g, vfvm.Physics("nlpoisson"))
    control = vfvm.SolverControl(precon_linear=precon, precision=precision, maxiters_linear=400, engine=engine)
    U = vfvm.solve(sys, inival=0.0, control=control)
    assert rel_err(U, oracle_solution(oracle, g, "nlpoisson", [])) <= SOL_TOL


@pytest.mark.parametrize("engine", ["persistent", "graph"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_porous_fixed_steps_vs_oracle(vfvm, oracle, precision, engine):
    g = vfvm.simplexgrid(lin(32), lin(32))
    x, y = g.coord
    u0 = 1e-3 + np.exp(-((x - 0.5) ** 2 + (y - 0.5) ** 2) / 0.1 ** 2)
    sys = vfvm.System(g, vfvm.Physics("porous"))
    control = vfvm.fixed_timesteps(vfvm.SolverControl(precision=precision, engine=engine), 1e-3)
    tsol = vfvm.solve(sys, inival=u0.reshape(1, -1), times=[0.0, 0.005], control=control)
    osys = oracle.OracleSystem(g, "porous")
    oc = oracle.fixed_timesteps(oracle.Control(), 1e-3)
    _, osols, _ = oracle.solve_transient(osys, u0, [0.0, 0.005], oc)
    assert len(tsol.u) == len(osols)
    assert rel_err(tsol.u[-1], osols[-1]) <= SOL_TOL


def test_rd2_vs_oracle(vfvm, oracle):
    g = vfvm.simplexgrid(lin(24), lin(24))
    params = [0.5, 2.0, 3.0]
    sys = vfvm.System(g, vfvm.Physics("rd2", params), species=[1, 2])
    U = vfvm.solve(sys, inival=0.5, control=vfvm.SolverControl(maxiters_linear=400))
    assert rel_err(U, oracle_solution(oracle, g, "rd2", params, inival=np.full(2 * g.nnodes, 0.5))) <= SOL_TOL


def test_kappa_exp_vs_oracle(vfvm, oracle):
    g = vfvm.simplexgrid(lin(24), lin(24))
    kappa = np.exp(np.random.default_rng(5).normal(size=g.nnodes))
    sys = vfvm.System(g, vfvm.Physics("kappa_exp", [0.7], kappa))
    U = vfvm.solve(sys, inival=0.0, control=vfvm.SolverControl(maxiters_linear=400))
    assert rel_err(U, oracle_solution(oracle, g, "kappa_exp", [0.7], nodedata=kappa)) <= SOL_TOL


@pytest.mark.parametrize("engine,precon", [("graph", "ilu0"), ("graph", "jacobi"), ("persistent", "ilu0"),
                                           ("persistent", "block_ilu0")])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_coarse_stage_vs_oracle(vfvm, oracle, engine, precon, precision):
    # the coarse-grid correction changes the Krylov iterations, not the solution
    g = vfvm.simplexgrid(lin(40), lin(40))
    kappa = np.exp(np.random.default_rng(6).normal(size=g.nnodes))
    sys = vfvm.System(g, vfvm.Physics("kappa_exp", [-0.4], kappa))
    plain = vfvm.SolverControl(engine=engine, precon_linear=precon, precision=precision, maxiters_linear=1000)
    vfvm.solve(sys, inival=0.0, control=plain)
    lin_plain = vfvm.solve.last_history.nlin
    control = vfvm.SolverControl(engine=engine, precon_linear=precon, precision=precision, maxiters_linear=1000,
                                 coarse=100)
    U = vfvm.solve(sys, inival=0.0, control=control)
    lin_coarse = vfvm.solve.last_history.nlin
    assert rel_err(U, oracle_solution(oracle, g, "kappa_exp", [-0.4], nodedata=kappa)) <= SOL_TOL
    assert lin_coarse < 0.7 * lin_plain


def test_bipolar_embedding_vs_oracle(vfvm, oracle):
    g = vfvm.simplexgrid(lin(6), lin(6), lin(6))
    sys = vfvm.System(g, vfvm.Physics("bipolar", BIPOLAR), species=[1, 2, 3])
    x = g.coord[0]
    C = np.where(x < 0.5, BIPOLAR[5], -BIPOLAR[5])
    nn = 0.5 * C + np.sqrt(0.25 * C * C + 1.0)
    inival = np.asfortranarray(np.stack([np.arcsinh(0.5 * C), nn, 1.0 / nn]))
    control = vfvm.SolverControl(precon_linear="ilu0", maxiters_linear=400, reltol_linear=1e-6)
    tsol = vfvm.solve(sys, inival=inival, embed=np.linspace(0.0, 1.0, 3), control=control)
    osys = oracle.OracleSystem(g, "bipolar", BIPOLAR)
    oc = oracle.Control()
    _, osols, _ = oracle.solve_transient(osys, inival.ravel(order="F"), np.linspace(0.0, 1.0, 3), oc, transient=False)
    assert rel_err(tsol.u[-1], osols[-1]) <= SOL_TOL


@pytest.mark.parametrize("precision,reltol_linear", [("fp64", 1e-6), ("mixed", 1e-3)])
def test_bipolar_fixed_ramp_block_jacobi_vs_oracle(vfvm, oracle, precision, reltol_linear):
    # the 3D drift-diffusion benchmark's form on a small grid: block-Jacobi (3x3)
    # BiCGStab, fixed embedding steps of 0.1 (no step control by the solution
    # change), FP32 Krylov refined by the FP64 Newton iteration in the mixed form
    g = vfvm.simplexgrid(lin(7), lin(7), lin(7))
    sys = vfvm.System(g, vfvm.Physics("bipolar", BIPOLAR), species=[1, 2, 3])
    C = np.where(g.coord[0] < 0.5, BIPOLAR[5], -BIPOLAR[5])
    nn = 0.5 * C + np.sqrt(0.25 * C * C + 1.0)
    inival = np.asfortranarray(np.stack([np.arcsinh(0.5 * C), nn, 1.0 / nn]))
    control = vfvm.SolverControl(precon_linear="jacobi", precision=precision, engine="graph", maxiters_linear=2000,
                                 reltol_linear=reltol_linear, updatecontrol=False, abstol=1e-10, reltol=0.0)
    control.Δp = control.Δp_max = control.Δp_min = 0.1
    control.Δu_opt = np.finfo(np.float64).max
    embed = np.linspace(0.0, 1.0, 11)
    tsol = vfvm.solve(sys, inival=inival, embed=embed, control=control)
    osys = oracle.OracleSystem(g, "bipolar", BIPOLAR)
    oc = oracle.Control()
    oc.Δp = oc.Δp_max = oc.Δp_min = 0.1
    oc.Δu_opt = np.finfo(np.float64).max
    _, osols, _ = oracle.solve_transient(osys, inival.ravel(order="F"), embed, oc, transient=False)
    assert rel_err(tsol.u[-1], osols[-1]) <= SOL_TOL


@pytest.mark.parametrize("dim,breg", [(2, 2), (3, 5)])
def test_surface_heat_steps_vs_oracle(vfvm, oracle, dim, breg):
    """Boundary fluxes, boundary storage and boundary sources through implicit
    Euler steps (device step control) against the oracle's fixed steps."""
    X = lin(16) if dim == 2 else lin(6)
    g = vfvm.simplexgrid(*([X] * dim))
    params = [1.0, 0.3, 0.5, 2.0, 10.0, breg]
    sys = vfvm.System(g, vfvm.Physics("surface_heat", params))
    u0 = np.full(g.nnodes, 0.2)
    control = vfvm.fixed_timesteps(vfvm.SolverControl(maxiters_linear=400, reltol_linear=1e-8), 0.02)
    tsol = vfvm.solve(sys, inival=u0.reshape(1, -1), times=[0.0, 0.1], control=control)
    osys = oracle.OracleSystem(g, "surface_heat", params)
    oc = oracle.fixed_timesteps(oracle.Control(), 0.02)
    _, osols, _ = oracle.solve_transient(osys, u0, [0.0, 0.1], oc)
    assert len(tsol.u) == len(osols) == 6
    assert rel_err(tsol.u[-1], osols[-1]) <= SOL_TOL
    assert np.max(tsol.u[-1]) > 0.2 + 1e-3  # the surface source warmed the layer above its start


@pytest.mark.parametrize("coarse", [0, 40])
def test_unstructured_grid_vs_oracle(vfvm, oracle, coarse):
    # Delaunay grid of a jittered lattice, read from a SimplexGrid text file
    g = vfvm.simplexgrid(os.path.join(GOLDEN, "jittered_square.sg"))
    kappa = np.exp(np.random.default_rng(9).normal(size=g.nnodes))
    sys = vfvm.System(g, vfvm.Physics("kappa_exp", [0.7], kappa))
    U = vfvm.solve(sys, inival=0.0, control=vfvm.SolverControl(maxiters_linear=400, coarse=coarse))
    assert rel_err(U, oracle_solution(oracle, g, "kappa_exp", [0.7], nodedata=kappa)) <= SOL_TOL


def test_convergence_error(vfvm):
    sys = vfvm.System(vfvm.simplexgrid(lin(16), lin(16)), vfvm.Physics("nlpoisson"))
    with pytest.raises(vfvm.ConvergenceError):
        vfvm.solve(sys, inival=0.0, maxiters=1)


@pytest.mark.parametrize("assembly", ["edgewise", "cellwise"])
@pytest.mark.parametrize("storage", ["dense", "sparse"])
def test_example210_two_species_transient(vfvm, testvals, assembly, storage):
    """examples/Example210_NonlinearPoisson2D_Reaction.jl: 100 implicit Euler
    steps of 0.01 on the device (step control on the device), sum of the
    last solution against the reference's testval, all four of its runtests
    combinations (:92-99)."""
    X = np.array([i / 10 for i in range(11)])
    sys = vfvm.System(vfvm.simplexgrid(X, X), vfvm.Physics("ex210", [1e-2, 1.0]), species=[1, 2],
                      assembly=assembly, unknown_storage=storage)
    control = vfvm.SolverControl(Δt=0.01, Δt_min=0.01, Δt_max=0.01, Δu_opt=1e5, reltol_linear=1e-10,
                                 maxiters_linear=400)
    tsol = vfvm.solve(sys, inival=0.0, times=[0.0, 1.0], control=control)
    assert float(np.sum(tsol.u[-1])) == pytest.approx(testvals["Example210_NonlinearPoisson2D_Reaction"]["value"],
                                                      rel=RTOL)
