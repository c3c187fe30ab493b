"""More of the reference's examples through the product API on the GPU, each
against the golden value in its runtests (tests/golden/reference_testvals.json)
with the solver tolerances each test states (tighter than the defaults where
the example's own tolerance asks for it):

* Example101: the 1D Laplace problem of the introduction (test030's system);
* Example102: three convection-diffusion fluxes (exponential, upwind, central);
* Example107: nonlinear storage with the adaptive step control on the device;
* Example115: a boundary species with mass-action boundary reactions and
  boundary storage, fixed steps, both storages and both catalytic ends;
* Example215: a boundary reaction between two bulk species, growing steps;
* Example220: a boundary species on a 2D grid with boundary storage.

The oracle restates the same examples (tests/test_oracle_golden.py);
Example220's GPU solution is also compared with the oracle's.
"""
import json
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN
from test_oracle_golden import barenblatt, ex115_system, ex215_inival, ex215_steps, ex220_steps, ex220_tables, lin

pytestmark = pytest.mark.gpu
RTOL = math.sqrt(np.finfo(float).eps)


@pytest.fixture(scope="module")
def testvals():
    with open(os.path.join(GOLDEN, "reference_testvals.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("assembly", ["edgewise", "cellwise"])
def test_example101_laplace(vfvm, testvals, assembly):
    """examples/Example101_Laplace1D.jl (runtests :126-129): -u'' = 0 on
    0:0.2:1, u = 0 and 1 at the ends by breaction penalties; sum(solution)."""
    g = vfvm.simplexgrid(np.array([k / 5 for k in range(6)]))
    sys = vfvm.System(g, vfvm.Physics("laplace_dirichlet"), assembly=assembly)
    U = vfvm.solve(sys, inival=0.0)
    assert float(U.sum()) == pytest.approx(testvals["Example101_Laplace1D"]["value"], rel=RTOL)


@pytest.mark.parametrize("assembly", ["edgewise", "cellwise"])
def test_example102_three_fluxes(vfvm, testvals, assembly):
    """examples/Example102_StationaryConvectionDiffusion1D.jl (runtests
    :138-141): D = 0.01, v = 1 on 0:0.1:1, u(0) = 0, u(1) = 1, from 0.5."""
    g = vfvm.simplexgrid(lin(10))
    total = 0.0
    for mode in (0, 1, 2):
        sys = vfvm.System(g, vfvm.Physics("ex102", [0.01, 1.0, mode]), assembly=assembly)
        vfvm.boundary_dirichlet(sys, 1, 1, 0.0)
        vfvm.boundary_dirichlet(sys, 1, 2, 1.0)
        U = vfvm.solve(sys, inival=vfvm.unknowns(sys, inival=0.5))
        total += float(U.sum())
    assert total == pytest.approx(testvals["Example102_StationaryConvectionDiffusion1D"]["value"], rel=RTOL)


@pytest.mark.parametrize("step_control", ["device", "host"])
@pytest.mark.parametrize("assembly", ["edgewise", "cellwise"])
def test_example107_nonlinear_storage(vfvm, testvals, assembly, step_control):
    """examples/Example107_NonlinearStorage1D.jl (runtests :118-124): storage
    (1e-10 + u)^(1/2) from the Barenblatt profile, t = 0.001 .. 0.01 under the
    adaptive step control (Δu_opt = 0.1, force_first_step); rtol 1e-5 as in the
    example (the oracle reproduces it in tests/test_oracle_golden.py)."""
    X = lin(20, -1.0, 1.0)
    g = vfvm.simplexgrid(X)
    sys = vfvm.System(g, vfvm.Physics("ex107", [2.0, 1e-10]), assembly=assembly)
    inival = np.array([barenblatt(x, 0.001, 2.0) ** 2.0 for x in X])
    control = vfvm.SolverControl(Δu_opt=0.1, force_first_step=True, step_control=step_control,
                                 reltol_linear=1e-10, maxiters_linear=400)
    tsol = vfvm.solve(sys, inival=inival[None, :], times=[0.001, 0.01], control=control)
    assert float(tsol.u[-1].sum()) == pytest.approx(testvals["Example107_NonlinearStorage1D"]["value"], rel=1e-5)


@pytest.mark.parametrize("storage", ["dense", "sparse"])
@pytest.mark.parametrize("assembly", ["edgewise", "cellwise"])
@pytest.mark.parametrize("switchbc", [False, True])
def test_example115_heterogeneous_catalysis(vfvm, testvals, assembly, storage, switchbc):
    """examples/Example115_HeterogeneousCatalysis1D.jl (runtests :223-233):
    species A, B in the bulk, C on the catalytic end, B = 0 at the other end;
    100 fixed steps of 0.01 with the step control on the device; u_C at the
    catalytic node at t = 1.  The example asks rtol 1e-12 of its direct
    solver; here BiCGStab runs to a relative 1e-12 in every Newton step, Newton
    to max|F| <= 1e-12, and the value meets 1e-10."""
    X, params, rs, bs, bf, bv, inodecat = ex115_system(vfvm, None, switchbc)
    icat, ibulk = (2, 1) if switchbc else (1, 2)
    sys = vfvm.System(vfvm.simplexgrid(X), vfvm.Physics("ex115", params), assembly=assembly,
                      unknown_storage=storage)
    vfvm.enable_species(sys, 1, [1])
    vfvm.enable_species(sys, 2, [1])
    vfvm.enable_boundary_species(sys, 3, [icat])
    vfvm.boundary_dirichlet(sys, 2, ibulk, 0.0)
    control = vfvm.fixed_timesteps(vfvm.SolverControl(abstol=1e-12, reltol=1e-12, reltol_linear=1e-12,
                                                      maxiters_linear=400), 0.01)
    tsol = vfvm.solve(sys, inival=0.0, times=[0.0, 1.0], control=control)
    assert len(tsol.t) == 101
    uc = float(tsol.u[-1][2, inodecat])
    assert uc == pytest.approx(testvals["Example115_HeterogeneousCatalysis1D"]["value"], rel=1e-10)
    # C lives only on the catalytic node: the other nodes keep 0 for it
    others = np.delete(np.arange(X.size), inodecat)
    assert np.all(tsol.u[-1][2, others] == 0.0)


@pytest.mark.parametrize("assembly", ["edgewise", "cellwise"])
def test_example215_boundary_reaction(vfvm, testvals, assembly):
    """examples/Example215_NonlinearPoisson2D_BoundaryReaction.jl (runtests
    :98-104): 42 implicit Euler steps of growing size, one solve call each;
    U[25] (species 1 of node 13)."""
    g = vfvm.simplexgrid(lin(10), lin(10))
    sys = vfvm.System(g, vfvm.Physics("ex215", [1.0e-2, 1.0]), assembly=assembly, species=[1, 2])
    U = ex215_inival(g).reshape(-1, 2).T.copy()
    control = vfvm.SolverControl(reltol_linear=1e-10, maxiters_linear=400)
    for dt in ex215_steps():
        U = vfvm.solve(sys, inival=U, control=control, tstep=dt)
    assert float(U[0, 12]) == pytest.approx(testvals["Example215_NonlinearPoisson2D_BoundaryReaction"]["value"],
                                            rel=RTOL)


@pytest.mark.parametrize("storage", ["dense", "sparse"])
def test_example220_boundary_species(vfvm, oracle, testvals, storage):
    """examples/Example220_NonlinearPoisson2D_BoundarySpecies.jl (runtests
    :100-104): species 3 on boundary region 2 (x = 1) with boundary storage
    and reactions, 100 steps of 0.01, one solve call each; species 3 at the
    fifth node of region 2.  The example's Newton reltol of 1e-5 is for its
    direct solver on this linear problem; the device solves to the default
    1e-10 with BiCGStab at 1e-10."""
    g = vfvm.simplexgrid(lin(10), lin(10))
    sys = vfvm.System(g, vfvm.Physics("ex220", [1.0, 1.0e-2]), unknown_storage=storage)
    vfvm.enable_species(sys, 1, [1])
    vfvm.enable_species(sys, 2, [1])
    vfvm.enable_boundary_species(sys, 3, [2])
    control = vfvm.SolverControl(reltol_linear=1e-10, maxiters_linear=400)
    U = vfvm.unknowns(sys, inival=0.0)
    for _ in range(ex220_steps()):
        U = vfvm.solve(sys, inival=U, control=control, tstep=0.01)
    r = np.sort(np.flatnonzero(np.abs(g.coord[0] - 1.0) < 1e-14))
    assert float(U[2, r[4]]) == pytest.approx(testvals["Example220_NonlinearPoisson2D_BoundarySpecies"]["value"],
                                              rel=RTOL)
    # against the oracle's solution, all three species
    rs, bs = ex220_tables()
    osys = oracle.OracleSystem(g, "ex220", [1.0, 1.0e-2], region_species=rs, bregion_species=bs)
    V = np.zeros(3 * g.nnodes)
    for _ in range(ex220_steps()):
        V, _ = oracle.solve_step(osys, V, oracle.Control(), 0.0, 0.01)
    Ud = np.asarray(U).T.ravel()
    assert np.max(np.abs(Ud - V)) <= 1e-8 * np.max(np.abs(V))
