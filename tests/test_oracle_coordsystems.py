"""Coordinate systems in the oracle: the checks of
examples/Example203_CoordinateSystems.jl (runtests :239-256), both assembly modes.

-div grad u = 1 on a disk (Polar1D), a cylinder (Cylindrical2D) and a ball
(Spherical1D) of radius 5 with u = 0 on the outer boundary: the discrete
solution equals the exact one, (r2^2 - r^2)/4 or /6, to 1e-14 (the example's
bound).  -div grad u = 0 on a ring, a cylinder shell and a spherical shell
between radii 1 and 5 with u = 1 inside and 0 outside: second order, max error
/ h^2 below 0.01 (ring, cylinder shell) and 0.04 (spherical shell).  The
example's unstructured cylinder reads a grid file of the reference's assets
and is not restated.  The form factors follow src/vfvm_formfactors.jl:25-62,
:102-161, :249-291.
"""
import math

import numpy as np
import pytest

H = 0.1
R1, R2 = 1.0, 5.0


def rng_(a, b):
    """Julia's collect(a:0.1:b), each value correctly rounded."""
    n = int(round((b - a) / H))
    return np.array([(10 * a + k) / 10 for k in range(n + 1)])


def ex203_case(vfvm, name):
    """(grid, source, Dirichlet values {region: value}, exact(r), bound, scaled) of one Example203 case."""
    if name == "disk":
        g = vfvm.circular_symmetric(vfvm.simplexgrid(rng_(0.0, R2)))
        return g, 1.0, {2: 0.0}, lambda r: 0.25 * (R2 ** 2 - r ** 2), 1e-14, False
    if name == "cylinder":
        g = vfvm.circular_symmetric(vfvm.simplexgrid(rng_(0.0, R2), rng_(0.0, 1.0)))
        return g, 1.0, {2: 0.0}, lambda r: 0.25 * (R2 ** 2 - r ** 2), 1e-14, False
    if name == "sphere":
        g = vfvm.spherical_symmetric(vfvm.simplexgrid(rng_(0.0, R2)))
        return g, 1.0, {2: 0.0}, lambda r: (R2 ** 2 - r ** 2) / 6.0, 1e-14, False
    if name == "ring":
        g = vfvm.circular_symmetric(vfvm.simplexgrid(rng_(R1, R2)))
        return g, 0.0, {1: 1.0, 2: 0.0}, lambda r: (np.log(r) - math.log(R2)) / (math.log(R1) - math.log(R2)), 0.01, True
    if name == "cylindershell":
        g = vfvm.circular_symmetric(vfvm.simplexgrid(rng_(R1, R2), rng_(0.0, 1.0)))
        return g, 0.0, {4: 1.0, 2: 0.0}, lambda r: (np.log(r) - math.log(R2)) / (math.log(R1) - math.log(R2)), 0.01, True
    if name == "sphereshell":
        g = vfvm.spherical_symmetric(vfvm.simplexgrid(rng_(R1, R2)))
        return g, 0.0, {1: 1.0, 2: 0.0}, lambda r: (R2 * R1 / r - R1) / (R2 - R1), 0.04, True
    raise KeyError(name)


CASES = ["disk", "cylinder", "sphere", "ring", "cylindershell", "sphereshell"]


def oracle_solve(vfvm, oracle, name, assembly):
    g, f, dirichlet, exact, bound, scaled = ex203_case(vfvm, name)
    nb = g.num_bfaceregions
    bf = np.zeros((1, nb)); bv = np.zeros((1, nb))
    for reg, val in dirichlet.items():
        bf[0, reg - 1] = 1e30
        bv[0, reg - 1] = val
    s = oracle.OracleSystem(g, "ex203", [f], bfactors=bf, bvalues=bv, assembly=assembly)
    u, _ = oracle.solve_step(s, np.zeros(g.nnodes), oracle.Control())
    return g, u, exact, bound, scaled


@pytest.mark.parametrize("assembly", ["edgewise", "cellwise"])
@pytest.mark.parametrize("name", CASES)
def test_example203_oracle(vfvm, oracle, name, assembly):
    g, u, exact, bound, scaled = oracle_solve(vfvm, oracle, name, assembly)
    err = np.max(np.abs(u - exact(g.coord[0])))
    assert (err / H ** 2 if scaled else err) < bound


def test_coordinate_system_volumes(vfvm, oracle):
    """The node volumes sum to the body's measure: disk pi r^2, ball 4/3 pi r^3,
    cylinder pi r^2 h (the boundary-face factors to its surface)."""
    for name, measure, bmeasure in [("disk", math.pi * R2 ** 2, None),
                                    ("sphere", 4.0 / 3.0 * math.pi * R2 ** 3, None),
                                    ("cylinder", math.pi * R2 ** 2, 2 * math.pi * R2 ** 2 + 2 * math.pi * R2)]:
        g = ex203_case(vfvm, name)[0]
        s = oracle.OracleSystem(g, "ex203", [1.0])
        assert s.nodevolumes().sum() == pytest.approx(measure, rel=1e-13)
        if bmeasure is not None:
            assert s.bfacefactors().sum() == pytest.approx(bmeasure, rel=1e-13)


def test_coordinate_system_validation(vfvm):
    with pytest.raises(ValueError):
        vfvm.spherical_symmetric(vfvm.simplexgrid(rng_(0.0, 1.0), rng_(0.0, 1.0)))
    with pytest.raises(ValueError):
        vfvm.circular_symmetric(vfvm.simplexgrid(rng_(0.0, 0.2), rng_(0.0, 0.2), rng_(0.0, 0.2)))
    g = vfvm.circular_symmetric(vfvm.simplexgrid(rng_(0.0, 1.0)))
    assert g.coordsystem == "polar1d" and "polar1d" in repr(g)
