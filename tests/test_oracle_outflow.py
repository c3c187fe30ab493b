"""Outflow boundaries (boutflow, src/vfvm_assembly.jl:239-313) in the oracle.

pluto-examples/outflow.jl's own checks in 1D, 2D and 3D: with the outflow
term the transported concentration stays at its inflow value c_in = 0.5
everywhere (max and min within Julia's isapprox), and the test-function
currents into and out of the domain balance (in = -out).
"""
import math

import numpy as np
import pytest

RTOL = math.sqrt(np.finfo(float).eps)


def outflow_case(vfvm, dim):
    X = np.array([i / 10 for i in range(11)])
    if dim == 1:
        return vfvm.simplexgrid(X), 1, 2
    if dim == 2:
        return vfvm.bfacemask(vfvm.simplexgrid(X, X), [1, 0.3], [1, 0.7], 5), 4, 5
    return vfvm.bfacemask(vfvm.simplexgrid(X, X, X), [0.3, 0.3, 0], [0.7, 0.7, 0], 7), 6, 7


def outflow_params(gin, gout):
    return [1.0, 1.0, 0.5, 1.0, gin, gout]  # k, v_in, c_in, D, G_in, G_out (FlowTransportData defaults)


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_oracle_outflow_example(vfvm, oracle, dim):
    g, gin, gout = outflow_case(vfvm, dim)
    o = oracle.OracleSystem(g, "outflow", outflow_params(gin, gout))
    sol, _ = oracle.solve_step(o, np.zeros(2 * g.nnodes), oracle.Control())
    c = sol.reshape(-1, 2)[:, 1]
    assert np.max(c) == pytest.approx(0.5, rel=RTOL) and np.min(c) == pytest.approx(0.5, rel=RTOL)
    tin = oracle.testfunction(g, [gout], [gin])
    tout = oracle.testfunction(g, [gin], [gout])
    Iin = o.integrate(tin, sol)["steady"]
    Iout = o.integrate(tout, sol)["steady"]
    assert np.allclose(Iin, -Iout, rtol=RTOL, atol=1e-12)
    assert Iin[0] == pytest.approx(1.0, rel=1e-10)  # v_in through a boundary of measure 1


def test_oracle_outflow_term_matters(vfvm, oracle):
    """Without the outflow term (no outflow region) the concentration is not constant."""
    g, gin, gout = outflow_case(vfvm, 2)
    U = np.stack([1.0 - g.coord[0], np.full(g.nnodes, 0.5)]).ravel(order="F")  # flow in +x
    o = oracle.OracleSystem(g, "outflow", outflow_params(gin, 99))  # no boundary region 99: no outflow nodes
    F, _ = o.assemble(U)
    o2 = oracle.OracleSystem(g, "outflow", outflow_params(gin, gout))
    F2, _ = o2.assemble(U)
    differ = np.flatnonzero(~np.isclose(F, F2))
    # only concentration rows: the p rows agree, since this state has p = 0 on the outflow region
    assert differ.size > 0 and np.all(differ % 2 == 1)
