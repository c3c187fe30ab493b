"""examples/Example161_BipolarDriftDiffusionCurrent.jl on the GPU.

The three adaptive transient phases run through the product API (the step
loop on the device); the test-function currents of the GPU's solutions are
taken twice: with the oracle's restatement of src/vfvm_testfunctions.jl, and
with the device's own test function and current integrals (the whole example
through the product API).  The step times must
equal the oracle's and the current sum the reference's testval within its own
tolerance (runtests :296-303, Julia's isapprox, rtol = sqrt(eps)).  Each
Newton step solves with BiCGStab to a relative 1e-12, so the Newton iterates
and their stopping decisions follow the direct solves of the reference.
"""
import math

import numpy as np
import pytest

import ex161_case as E

pytestmark = pytest.mark.gpu
RTOL = math.sqrt(np.finfo(float).eps)


@pytest.mark.parametrize("step_control", ["device", "host"])
def test_example161_current_gpu(vfvm, oracle, step_control):
    import json, os
    from conftest import GOLDEN
    with open(os.path.join(GOLDEN, "reference_testvals.json")) as f:
        ref = json.load(f)["Example161_BipolarDriftDiffusionCurrent"]["value"]
    g = E.grid(vfvm)
    sys = vfvm.System(g, vfvm.Physics("ex161", E.PARAMS))
    base, phases = E.control_fields()
    control = vfvm.SolverControl(reltol_linear=1e-12, maxiters_linear=400, step_control=step_control,
                                 Δu_opt=math.inf, **base)
    u = E.inival(E.coords())
    for (t0, t1), fields in phases:
        for k, v in fields.items():
            setattr(control, k, v)
        tsol = vfvm.solve(sys, inival=u, times=[t0, t1], control=control)
        u = tsol.u[-1]
    # the oracle's step times of the last phase
    osys = oracle.OracleSystem(g, "ex161", E.PARAMS)
    c = oracle.Control()
    c.Δu_opt = math.inf
    for k, v in base.items():
        setattr(c, k, v)
    uo = E.inival(E.coords()).ravel(order="F")
    for (t0, t1), fields in phases:
        for k, v in fields.items():
            setattr(c, k, v)
        otimes, osols, _ = oracle.solve_transient(osys, uo, [t0, t1], c)
        uo = osols[-1]
    assert np.allclose(tsol.t, otimes, rtol=1e-14, atol=0)
    sols = [np.asarray(x).ravel(order="F") for x in tsol.u]
    assert max(np.max(np.abs(a - b)) for a, b in zip(sols, osols)) <= 1e-8
    tf = oracle.testfunction(g, [1], [2])
    assert E.current_sum(osys, tf, tsol.t, sols) == pytest.approx(ref, rel=RTOL)
    # the whole example through the product API: the device test function and currents
    T = vfvm.testfunction(vfvm.TestFunctionFactory(sys), [1], [2])
    total = 0.0
    for k in range(1, len(tsol.t)):
        dt = tsol.t[k] - tsol.t[k - 1]
        e_new = vfvm.integrate_gradT_flux(sys, T, tsol.u[k])
        e_old = vfvm.integrate_gradT_flux(sys, T, tsol.u[k - 1])
        total += e_new[0] + e_new[1] + (e_new[2] - e_old[2]) / dt
    assert total == pytest.approx(ref, rel=RTOL)
