"""Parameter derivatives of the residual (the reference's dudp) on the GPU.

* ``parameter_derivatives`` against the oracle's restatement of the asm_param
  accumulation (src/vfvm_assembly.jl:116-120,194-198,403-405), within 1e-12 of
  each row's scale, in both assembly modes of the oracle;
* examples/Example430_ParameterDerivativesStationary.jl (runh) with the GPU's
  solves, Jacobians and dudp: the sum of dm/dp over p in 0.1:0.05:2 meets the
  reference's testval within its own tolerance (Julia's isapprox, sqrt(eps)).
  The current m and its derivatives dm/du, dm/dp are post-processing of the
  solution; they come from the oracle's restatement of the test functions.
"""
import math

import numpy as np
import pytest
import scipy.sparse.linalg as spla

from gpu_cases import lin

pytestmark = pytest.mark.gpu
RTOL = math.sqrt(np.finfo(float).eps)


@pytest.mark.parametrize("n", [10, 32])
@pytest.mark.parametrize("assembly", ["edgewise", "cellwise"])
def test_parameter_derivatives_vs_oracle(vfvm, oracle, n, assembly):
    g = vfvm.simplexgrid(lin(n), lin(n))
    p = 0.7
    sys = vfvm.System(g, vfvm.Physics("ex430", [p]), assembly=assembly)
    osys = oracle.OracleSystem(g, "ex430", [p], assembly=assembly)
    U = np.random.default_rng(n).uniform(0.2, 1.0, g.nnodes)
    d = vfvm.parameter_derivatives(sys, U.reshape(1, -1))
    assert d.shape == (1, 1, g.nnodes)
    do = osys.parameter_derivatives(U)
    scale = np.maximum(np.abs(do[0]), 1.0)
    assert np.all(np.abs(d[0].ravel() - do[0]) <= 1e-12 * scale)
    # a physics without differentiable parameters has none
    assert vfvm.parameter_derivatives(vfvm.System(g, vfvm.Physics("nlpoisson")), np.zeros(g.nnodes)).shape[0] == 0


def test_example430_on_gpu(vfvm, oracle):
    import json, os
    from conftest import GOLDEN
    with open(os.path.join(GOLDEN, "reference_testvals.json")) as f:
        ref = json.load(f)["Example430_ParameterDerivativesStationary"]["value"]
    X = np.array([i / 10 for i in range(11)])
    g = vfvm.simplexgrid(X, X)
    T = oracle.testfunction(g, [1], [3])
    control = vfvm.SolverControl(reltol_linear=1e-12, maxiters_linear=400)
    total = 0.0
    for k in range(39):
        p = 0.1 + 0.05 * k
        sys = vfvm.System(g, vfvm.Physics("ex430", [p]))
        sol = vfvm.solve(sys, inival=0.5, control=control)
        _, J = vfvm.evaluate_residual_and_jacobian(sys, sol)
        dFdp = vfvm.parameter_derivatives(sys, sol)[0].ravel()
        du, dp = oracle.OracleSystem(g, "ex430", [p]).integrate_gradient(T, sol.ravel())
        total += -du @ spla.splu(J.tocsc()).solve(dFdp) + dp[0]
        sys.close()
    assert total == pytest.approx(ref, rel=RTOL)
