"""Pin the CPU oracle against the reference's own golden values and unit tests.

Each case restates a reference example (physics in oracle/vfvm_oracle.cpp, driver
here) and compares with the `testval` recorded in the example
(tests/golden/reference_testvals.json, generated from the reference sources by
tests/golden/make_fixtures.py).  Tolerance: Julia's default isapprox
(rtol = sqrt(eps)) unless the example states another one.
"""
import json
import math
import os

import numpy as np
import pytest
import scipy.sparse.linalg as spla

from conftest import GOLDEN

RTOL = math.sqrt(np.finfo(float).eps)


@pytest.fixture(scope="module")
def testvals():
    with open(os.path.join(GOLDEN, "reference_testvals.json")) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def grid(vfvm):
    return vfvm.simplexgrid


def lin(n, a=0.0, b=1.0):
    # the values of Julia's range a:(b-a)/n:b, each correctly rounded
    return np.array([a + (b - a) * i / n for i in range(n + 1)]) if a == 0.0 else np.array([(a * n + (b - a) * i) / n for i in range(n + 1)])


def test_example105(oracle, grid, testvals):
    g = grid(lin(10))
    bf = np.full((1, 2), 1e30)
    bv = np.array([[0.0, 1.0]])
    s = oracle.OracleSystem(g, "ex105", [1e-3], bfactors=bf, bvalues=bv)
    u, _ = oracle.solve_step(s, np.full(g.nnodes, 0.5), oracle.Control())
    assert u.sum() == pytest.approx(testvals["Example105_NonlinearPoisson1D"]["value"], rel=RTOL)


def barenblatt(x, t, m):
    tx = t ** (-1.0 / (m + 1.0))
    xx = x * tx
    xx = xx * xx
    xx = 1 - xx * (m - 1) / (2.0 * m * (m + 1))
    xx = max(xx, 0.0)
    return tx * xx ** (1.0 / (m - 1.0))


def test_example106_transient(oracle, grid, testvals):
    X = np.array([(i - 10) / 10 for i in range(21)])
    g = grid(X)
    s = oracle.OracleSystem(g, "ex106", [2.0])
    c = oracle.Control()
    c.Δt_min = c.Δt_max = c.Δt = 1e-4
    c.Δu_opt = 1.0
    ts, sols, _ = oracle.solve_transient(s, np.array([barenblatt(x, 0.001, 2.0) for x in X]), [0.001, 0.01], c)
    assert sols[-1].sum() == pytest.approx(testvals["Example106_NonlinearDiffusion1D"]["value"], rel=RTOL)


def test_example110_two_species(oracle, grid, testvals):
    g = grid(lin(100))
    bf = np.full((2, 2), 1e30)
    bv = np.array([[1.0, 0.0], [1.0, 0.0]])
    U = np.zeros(2 * g.nnodes)
    c = oracle.Control()
    c.damp_initial = 0.1
    for xeps in [1.0, 0.5, 0.25, 0.1, 0.05, 0.025, 0.01]:
        s = oracle.OracleSystem(g, "ex110", [xeps, xeps], bfactors=bf, bvalues=bv)
        U, _ = oracle.solve_step(s, U, c)
    assert U[4] == pytest.approx(testvals["Example110_ReactionDiffusion1D_TwoSpecies"]["value"], rel=RTOL)


def test_example160_bernoulli_sedan(oracle, grid, testvals):
    g = grid(lin(20))
    s = oracle.OracleSystem(g, "ex160", [1e-3, -1.0, 5.0])
    c = oracle.Control()
    c.Δt_min = 1e-5; c.Δt = 1e-5; c.Δt_grow = 1.1; c.Δt_max = 0.1; c.Δu_opt = 0.1; c.damp_initial = 0.5
    inival = np.zeros(2 * g.nnodes)
    inival[1::2] = 0.5
    ts, sols, _ = oracle.solve_transient(s, inival, [0.0, 10.0], c)
    # examples/Example160_UnipolarDriftDiffusion1D.jl:262: rtol = 1e-5
    assert sols[-1].sum() == pytest.approx(testvals["Example160_UnipolarDriftDiffusion1D"]["value"], rel=1e-5)


def test_example207_2d_timesteps(oracle, grid, testvals):
    g = grid(lin(10), lin(10))
    bf = np.zeros((1, 4)); bv = np.zeros((1, 4))
    bf[0, 1] = bf[0, 3] = 1e30
    bv[0, 1] = bv[0, 3] = 0.1
    s = oracle.OracleSystem(g, "ex207", [1e-2], bfactors=bf, bvalues=bv)
    inival = np.full(g.nnodes, 0.5)
    t = 0.0
    while t < 1.0:
        t = t + 0.01
        U, _ = oracle.solve_step(s, inival, oracle.Control(), 0.0, 0.01)
        inival = U.copy()
    assert U[14] == pytest.approx(testvals["Example207_NonlinearPoisson2D"]["value"], rel=RTOL)


def test_example301_3d(oracle, grid, testvals):
    g = grid(lin(5), lin(5), lin(5))
    bf = np.zeros((1, 6)); bv = np.zeros((1, 6))
    bf[0, 4] = bf[0, 5] = 1e30
    s = oracle.OracleSystem(g, "ex301", [], bfactors=bf, bvalues=bv)
    u, _ = oracle.solve_step(s, np.zeros(g.nnodes), oracle.Control())
    assert u[42] == pytest.approx(testvals["Example301_Laplace3D"]["value"], rel=RTOL)


def test_example440_many_instances(oracle, grid, testvals):
    g = grid(np.array([i / 320 for i in range(321)]))
    total = 0.0
    for i in range(100):
        s = oracle.OracleSystem(g, "ex440", [i * 10.0 / 99.0])
        c = oracle.Control()
        c.abstol = 1e-15
        c.reltol = 1e-20
        u, _ = oracle.solve_step(s, np.full(g.nnodes, 0.1), c)
        total += float(np.dot(s.nodevolumes(), u))
    assert total == pytest.approx(testvals["Example440_ParallelState"]["value"], rel=RTOL)


def test_cachesol_linear_exact(oracle, grid):
    # test/test030_cachesol.jl: 1D Laplace, solution equals x.  The reference pins
    # 3e-16 with UMFPACK; SuperLU (the stand-in direct solver) gives a few ulps.
    X = np.array([i / 9 for i in range(10)])
    s = oracle.OracleSystem(grid(X), "laplace_dirichlet")
    F, J = s.assemble(np.zeros(10))
    x = s.linsolve(J, -F)
    assert np.max(np.abs(x - X)) <= 1e-15


@pytest.mark.parametrize("assembly", ["edgewise", "cellwise"])
def test_example161_current(vfvm, oracle, testvals, assembly):
    """Example161: bipolar drift-diffusion in three cell regions, three adaptive
    transient phases, test-function current integrals (runtests :296-303)."""
    import ex161_case as E
    g = E.grid(vfvm)
    osys = oracle.OracleSystem(g, "ex161", E.PARAMS, assembly=assembly)
    c = oracle.Control()
    c.Δu_opt = math.inf
    base, phases = E.control_fields()
    for k, v in base.items():
        setattr(c, k, v)
    u = E.inival(E.coords()).ravel(order="F")
    for (t0, t1), fields in phases:
        for k, v in fields.items():
            setattr(c, k, v)
        times, sols, _ = oracle.solve_transient(osys, u, [t0, t1], c)
        u = sols[-1]
    tf = oracle.testfunction(g, [1], [2], assembly=assembly)
    assert len(times) == 119
    ref = testvals["Example161_BipolarDriftDiffusionCurrent"]["value"]
    assert E.current_sum(osys, tf, times, sols) == pytest.approx(ref, rel=RTOL)


def ex430_sum(vfvm, oracle, solve_and_derivatives):
    """Example430's runh (:183-247): for p in 0.1:0.05:2 the steady current m
    between boundary regions 1 and 3 and its total derivative
    dm/dp = -dm/du (J \\ dudp) + dm/dp; the sum over p."""
    X = np.array([i / 10 for i in range(11)])
    g = vfvm.simplexgrid(X, X)
    T = oracle.testfunction(g, [1], [3])
    total = 0.0
    for k in range(39):
        p = 0.1 + 0.05 * k
        osys = oracle.OracleSystem(g, "ex430", [p])
        sol, J, dFdp = solve_and_derivatives(g, p, osys)
        du, dp = osys.integrate_gradient(T, sol)
        total += -du @ spla.splu(J.tocsc()).solve(dFdp) + dp[0]
    return total


def test_example430_parameter_derivatives(vfvm, oracle, testvals):
    """Example430 (runtests :250-257): parameter derivatives of a stationary
    solve through dudp, the Jacobian and the test-function current."""
    def oracle_solve(g, p, osys):
        sol, _ = oracle.solve_step(osys, np.full(g.nnodes, 0.5), oracle.Control())
        _, J = osys.assemble(sol)
        return sol, J, osys.parameter_derivatives(sol)[0]
    ref = testvals["Example430_ParameterDerivativesStationary"]["value"]
    assert ex430_sum(vfvm, oracle, oracle_solve) == pytest.approx(ref, rel=RTOL)


def test_oracle_parameter_derivatives_vs_differences(vfvm, oracle):
    """dudp against central differences of the residual in p."""
    X = np.array([i / 10 for i in range(11)])
    g = vfvm.simplexgrid(X, X)
    U = np.random.default_rng(2).uniform(0.2, 1.0, g.nnodes)
    p, h = 0.7, 1e-6
    d = oracle.OracleSystem(g, "ex430", [p]).parameter_derivatives(U)[0]
    Fp, _ = oracle.OracleSystem(g, "ex430", [p + h]).assemble(U)
    Fm, _ = oracle.OracleSystem(g, "ex430", [p - h]).assemble(U)
    fd = (Fp - Fm) / (2 * h)
    # rows of the Dirichlet nodes carry the 1e30 penalty, where differences of F
    # only resolve the penalty's own derivative (regions 3: -1e30 * factor)
    dirichlet = np.zeros(g.nnodes, dtype=bool)
    dirichlet[np.unique(g.bfacenodes[:, np.isin(g.bfaceregions, [1, 3])])] = True
    assert np.allclose(d[~dirichlet], fd[~dirichlet], rtol=1e-6, atol=1e-8)
    big = np.abs(d) > 1e20
    assert big.any() and np.allclose(d[big], fd[big], rtol=1e-6)


def ex210_grid(vfvm):
    X = np.array([i / 10 for i in range(11)])  # range(0, 1, length = 11)
    return vfvm.simplexgrid(X, X)


@pytest.mark.parametrize("assembly", ["edgewise", "cellwise"])
def test_example210_transient(vfvm, oracle, testvals, assembly):
    """Example210 (runtests :92-99): two-species reaction-diffusion, 100
    implicit Euler steps of 0.01 (Δt_min = Δt_max = Δt, Δu_opt = 1e5)."""
    g = ex210_grid(vfvm)
    osys = oracle.OracleSystem(g, "ex210", [1e-2, 1.0], assembly=assembly)
    c = oracle.Control()
    c.Δt = c.Δt_min = c.Δt_max = 0.01
    c.Δu_opt = 1e5
    times, sols, _ = oracle.solve_transient(osys, np.zeros(2 * g.nnodes), [0.0, 1.0], c)
    ref = testvals["Example210_NonlinearPoisson2D_Reaction"]["value"]
    assert float(np.sum(sols[-1])) == pytest.approx(ref, rel=RTOL)


@pytest.mark.parametrize("assembly", ["edgewise", "cellwise"])
def test_example101_laplace(vfvm, oracle, testvals, assembly):
    """Example101 (runtests :126-129): -u'' = 0 on 0:0.2:1 with the breaction
    penalties u = 0 on region 1 and u = 1 on region 2 (test030's system); the
    sum of the solution."""
    g = vfvm.simplexgrid(np.array([k / 5 for k in range(6)]))
    s = oracle.OracleSystem(g, "laplace_dirichlet", assembly=assembly)
    u, _ = oracle.solve_step(s, np.zeros(g.nnodes), oracle.Control())
    assert float(u.sum()) == pytest.approx(testvals["Example101_Laplace1D"]["value"], rel=RTOL)


def test_example102_three_fluxes(vfvm, oracle, testvals):
    """Example102 (runtests :138-141): the exponential, upwind and central
    fluxes on 0:0.1:1, u(0) = 0, u(1) = 1, from 0.5; the sum of the three
    solutions."""
    g = vfvm.simplexgrid(lin(10))
    bf = np.full((1, 2), 1e30)
    bv = np.array([[0.0, 1.0]])
    total = 0.0
    for mode in (0, 1, 2):
        s = oracle.OracleSystem(g, "ex102", [0.01, 1.0, mode], bfactors=bf, bvalues=bv, assembly="cellwise")
        u, _ = oracle.solve_step(s, np.full(g.nnodes, 0.5), oracle.Control())
        total += float(u.sum())
    assert total == pytest.approx(testvals["Example102_StationaryConvectionDiffusion1D"]["value"], rel=RTOL)


@pytest.mark.parametrize("assembly", ["edgewise", "cellwise"])
def test_example107_nonlinear_storage(vfvm, oracle, testvals, assembly):
    """Example107 (runtests :118-124): storage (1e-10 + u)^(1/2) from the
    Barenblatt profile at t = 0.001 to t = 0.01 with the adaptive step control
    (Δu_opt = 0.1, force_first_step), rtol 1e-5 as in the example."""
    X = lin(20, -1.0, 1.0)
    s = oracle.OracleSystem(vfvm.simplexgrid(X), "ex107", [2.0, 1e-10], assembly=assembly)
    c = oracle.Control()
    c.Δu_opt = 0.1
    c.force_first_step = True
    inival = np.array([barenblatt(x, 0.001, 2.0) ** 2.0 for x in X])
    _, sols, _ = oracle.solve_transient(s, inival, [0.001, 0.01], c)
    assert float(sols[-1].sum()) == pytest.approx(testvals["Example107_NonlinearStorage1D"]["value"], rel=1e-5)


def ex115_system(vfvm, oracle_or_none, switchbc, assembly="edgewise"):
    """Grid, parameters and species tables of Example115 (main, :82-170)."""
    X = lin(10)
    icat, ibulk, inodecat = (2, 1, X.size - 1) if switchbc else (1, 2, 0)
    params = [1.0, 1.0e-2, 100.0, 1.0, 0.1, 1.0, 0.01, icat]
    rs = np.array([[1], [1], [0]])
    bs = np.zeros((3, 2), dtype=int)
    bs[2, icat - 1] = 1
    bf = np.zeros((3, 2)); bv = np.zeros((3, 2))
    bf[1, ibulk - 1] = 1e30          # boundary_dirichlet!(sys, iB, iBulk, 0.0)
    return X, params, rs, bs, bf, bv, inodecat


@pytest.mark.parametrize("assembly", ["edgewise", "cellwise"])
@pytest.mark.parametrize("switchbc", [False, True])
def test_example115_heterogeneous_catalysis(vfvm, oracle, testvals, assembly, switchbc):
    """Example115 (runtests :223-233): boundary species C on the catalytic end
    (mass-action breaction, bstorage), B = 0 at the other end, 100 fixed steps
    of 0.01; u_C at the catalytic node at t = 1, rtol 1e-12 as in the example."""
    X, params, rs, bs, bf, bv, inodecat = ex115_system(vfvm, oracle, switchbc)
    s = oracle.OracleSystem(vfvm.simplexgrid(X), "ex115", params, bfactors=bf, bvalues=bv, assembly=assembly,
                            region_species=rs, bregion_species=bs)
    c = oracle.fixed_timesteps(oracle.Control(), 0.01)
    _, sols, _ = oracle.solve_transient(s, np.zeros(3 * X.size), [0.0, 1.0], c)
    uc = sols[-1][3 * inodecat + 2]
    assert uc == pytest.approx(testvals["Example115_HeterogeneousCatalysis1D"]["value"], rel=1e-12)


def ex215_inival(g):
    x, y = g.coord[0], g.coord[1]
    U = np.zeros(2 * g.nnodes)
    U[0::2] = np.exp(-5.0 * ((x - 0.5) ** 2 + (y - 0.5) ** 2))
    return U


def ex215_steps():
    """The example's time loop (:69-75): tstep from 0.01, times 1.2 per step, until time >= 100."""
    steps, time, tstep = [], 0.0, 0.01
    while time < 100.0:
        time = time + tstep
        steps.append(tstep)
        tstep *= 1.2
    return steps


@pytest.mark.parametrize("assembly", ["edgewise", "cellwise"])
def test_example215_boundary_reaction(vfvm, oracle, testvals, assembly):
    """Example215 (runtests :98-104): two species exchanged by a boundary
    reaction on region 2, 42 growing implicit Euler steps; U[25] (species 1 of
    node 13)."""
    g = vfvm.simplexgrid(lin(10), lin(10))
    s = oracle.OracleSystem(g, "ex215", [1.0e-2, 1.0], assembly=assembly)
    U = ex215_inival(g)
    for dt in ex215_steps():
        U, _ = oracle.solve_step(s, U, oracle.Control(), 0.0, dt)
    assert U[24] == pytest.approx(testvals["Example215_NonlinearPoisson2D_BoundaryReaction"]["value"], rel=RTOL)


def ex220_tables():
    rs = np.array([[1], [1], [0]])
    bs = np.zeros((3, 4), dtype=int)
    bs[2, 1] = 1
    return rs, bs


def ex220_steps():
    """The example's time loop (:77-83): tstep 0.01 while time < 1."""
    n, time = 0, 0.0
    while time < 1.0:
        time = time + 0.01
        n += 1
    return n


def ex220_u5(g, U):
    """U_bound[5]: species 3 on the fifth node of boundary region 2 (x = 1),
    the subgrid's nodes in the order of their parent indices."""
    r = np.flatnonzero(np.abs(g.coord[0] - 1.0) < 1e-14)
    return U[3 * np.sort(r)[4] + 2]


@pytest.mark.parametrize("assembly", ["edgewise", "cellwise"])
def test_example220_boundary_species(vfvm, oracle, testvals, assembly):
    """Example220 (runtests :100-104): bulk species 1, 2 and species 3 on
    boundary region 2 (bstorage, breaction), 100 steps of 0.01 with Newton
    reltol 1e-5; species 3 at the fifth node of region 2."""
    g = vfvm.simplexgrid(lin(10), lin(10))
    rs, bs = ex220_tables()
    s = oracle.OracleSystem(g, "ex220", [1.0, 1.0e-2], assembly=assembly, region_species=rs, bregion_species=bs)
    c = oracle.Control()
    c.reltol = 1e-5
    U = np.zeros(3 * g.nnodes)
    for _ in range(ex220_steps()):
        U, _ = oracle.solve_step(s, U, c, 0.0, 0.01)
    assert ex220_u5(g, U) == pytest.approx(testvals["Example220_NonlinearPoisson2D_BoundarySpecies"]["value"],
                                           rel=RTOL)
