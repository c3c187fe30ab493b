"""Outflow boundaries (boutflow, src/vfvm_assembly.jl:239-313) on the GPU:
pluto-examples/outflow.jl through the product API in 1D, 2D and 3D against
the oracle (1e-8 relative) and the example's own checks (constant
concentration c_in, balanced test-function currents).  Assembly parity of the
outflow physics runs with the other physics in test_gpu_assembly.py."""
import math

import numpy as np
import pytest

from test_oracle_outflow import outflow_case, outflow_params

pytestmark = pytest.mark.gpu
RTOL = math.sqrt(np.finfo(float).eps)


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_outflow_example_gpu(vfvm, oracle, dim):
    g, gin, gout = outflow_case(vfvm, dim)
    sys = vfvm.System(g, vfvm.Physics("outflow", outflow_params(gin, gout)))
    sol = vfvm.solve(sys, inival=0.0, control=vfvm.SolverControl(reltol_linear=1e-12, maxiters_linear=400))
    o = oracle.OracleSystem(g, "outflow", outflow_params(gin, gout))
    uo, _ = oracle.solve_step(o, np.zeros(2 * g.nnodes), oracle.Control())
    assert np.max(np.abs(sol.ravel(order="F") - uo)) <= 1e-8 * np.max(np.abs(uo))
    assert np.max(sol[1]) == pytest.approx(0.5, rel=RTOL) and np.min(sol[1]) == pytest.approx(0.5, rel=RTOL)
    tf = vfvm.TestFunctionFactory(sys)
    Iin = vfvm.integrate(sys, vfvm.testfunction(tf, [gout], [gin]), sol)
    Iout = vfvm.integrate(sys, vfvm.testfunction(tf, [gin], [gout]), sol)
    assert np.allclose(Iin, -Iout, rtol=1e-8, atol=1e-10)
