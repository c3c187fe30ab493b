"""Coordinate systems on the GPU (examples/Example203_CoordinateSystems.jl): the
product's form factors for polar and spherical 1D and cylindrical 2D grids
against the oracle's restatement of src/vfvm_formfactors.jl, and Example203's
six cases solved through the product API.

The example asks the disk, cylinder and ball solutions to equal the exact
ones to 1e-14, which its direct solver reaches; here BiCGStab runs to a
relative 1e-12 per Newton step, so those three are checked against the exact
solution to 1e-9 of its maximum, every case against the oracle's solution to
1e-8 (the solution-parity bar), and the shells against the example's own
second-order bounds.
"""
import numpy as np
import pytest

from test_oracle_coordsystems import CASES, H, ex203_case, oracle_solve

pytestmark = pytest.mark.gpu


def product_system(vfvm, name, assembly="edgewise"):
    g, f, dirichlet, exact, bound, scaled = ex203_case(vfvm, name)
    sys = vfvm.System(g, vfvm.Physics("ex203", [f]), assembly=assembly)
    for reg, val in dirichlet.items():
        vfvm.boundary_dirichlet(sys, 1, reg, val)
    return g, sys, exact, bound, scaled


@pytest.mark.parametrize("name", CASES)
def test_coordsystem_factors(vfvm, oracle, name):
    g, sys, _, _, _ = product_system(vfvm, name)
    nv = vfvm.nodevolumes(sys)
    ef, en = vfvm.edgefactors(sys)
    nvo, efo, eno = oracle.OracleSystem(g, "ex203", [1.0]).factors()
    assert np.array_equal(en, eno)
    np.testing.assert_allclose(nv, nvo, rtol=1e-13, atol=1e-16)
    np.testing.assert_allclose(ef, efo, rtol=1e-12, atol=1e-14 * np.max(np.abs(efo)))


@pytest.mark.parametrize("assembly", ["edgewise", "cellwise"])
@pytest.mark.parametrize("name", CASES)
def test_example203_gpu(vfvm, oracle, name, assembly):
    g, sys, exact, bound, scaled = product_system(vfvm, name, assembly)
    control = vfvm.SolverControl(reltol_linear=1e-12, maxiters_linear=1000)
    U = vfvm.solve(sys, inival=0.0, control=control)
    u = np.asarray(U)[0]
    _, uo, _, _, _ = oracle_solve(vfvm, oracle, name, assembly)
    assert np.max(np.abs(u - uo)) <= 1e-8 * np.max(np.abs(uo))
    ue = exact(g.coord[0])
    err = np.max(np.abs(u - ue))
    if scaled:
        assert err / H ** 2 < bound
    else:
        assert err <= 1e-9 * np.max(np.abs(ue))
