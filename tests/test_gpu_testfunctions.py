"""Test-function currents on the GPU (src/vfvm_testfunctions.jl:38-380) against
the oracle's restatement.

* ``vfvm_integrate``: the six per-species sums (flux, reaction, source,
  storage of U and of Uold, edge reaction) at random states, within 1e-10 of
  the oracle's (the sums are taken in another order);
* ``testfunction``: the Laplace solve with T = 0 / 1 on the chosen boundary
  regions, within 1e-10 of the oracle's direct solve.
"""
import numpy as np
import pytest

from gpu_cases import case, random_state

pytestmark = pytest.mark.gpu
PARTS = ("flux", "react", "src", "stor", "oldstor", "erea")


@pytest.mark.parametrize("name", ["ex161", "kappa_exp", "edge_reaction2d", "bipolar", "surface_heat2d", "rd2"])
def test_integrals_vs_oracle(vfvm, oracle, name):
    c = case(vfvm, name)
    sys = vfvm.System(c["grid"], vfvm.Physics(c["kind"], c["params"], c["nodedata"]))
    osys = oracle.OracleSystem(c["grid"], c["kind"], c["params"], nodedata=c["nodedata"])
    rng = np.random.default_rng(17)
    U = random_state(c, sys.nspec, rng)
    Uold = random_state(c, sys.nspec, rng)
    T = rng.uniform(0.0, 1.0, c["grid"].nnodes)
    gpu = vfvm.system._tf_parts(sys, T, U, Uold)
    ref = osys.integrate(T, U.ravel(order="F"), Uold.ravel(order="F"))
    for k in PARTS:
        scale = max(1.0, float(np.max(np.abs(ref[k]))))
        assert np.allclose(gpu[k], ref[k], rtol=1e-10, atol=1e-10 * scale), k
    # the composed forms of the reference
    steady = vfvm.integrate(sys, T, U)
    assert np.allclose(steady, ref["flux"] + ref["react"] - ref["src"] + ref["erea"], rtol=1e-10,
                       atol=1e-10 * max(1.0, float(np.max(np.abs(steady)))))
    assert np.allclose(vfvm.integrate_gradT_flux(sys, T, U), ref["flux"], rtol=1e-10,
                       atol=1e-10 * max(1.0, float(np.max(np.abs(ref["flux"])))))


@pytest.mark.parametrize("name", ["ex161", "kappa_exp", "surface_heat3d"])
def test_testfunction_vs_oracle(vfvm, oracle, name):
    c = case(vfvm, name)
    g = c["grid"]
    sys = vfvm.System(g, vfvm.Physics(c["kind"], c["params"], c["nodedata"]))
    bc0, bc1 = [1], [2]
    T = vfvm.testfunction(vfvm.TestFunctionFactory(sys), bc0, bc1)
    To = oracle.testfunction(g, bc0, bc1)
    assert np.max(np.abs(T - To)) <= 1e-10
    assert np.min(T) >= -1e-10 and np.max(T) <= 1 + 1e-10
