"""Edge reactions (src/vfvm_assembly.jl:202-238) on the GPU, through the C ABI.

Assembly parity of the edge-reaction physics runs with the other physics in
test_gpu_assembly.py (cases edge_reaction2d, edge_reaction3d, joule_heat).
Here: examples/DevEx002_EdgeReaction.jl's own check (runtests :181-205,
case :compare_max) through the product API in 1D, 2D and 3D, and Newton
solves against the oracle (1e-8 relative, the solve tolerance of the other
solution tests).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
SOL_TOL = 1e-8


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_devex002_compare_max_gpu(vfvm, oracle, dim):
    X = np.arange(0.0, 1.0 + 1e-12, 0.25)
    g = vfvm.simplexgrid(*([X] * dim))
    control = vfvm.SolverControl(reltol_linear=1e-12, maxiters_linear=400)
    mx = []
    for mode in (0, 1, 2):
        sys = vfvm.System(g, vfvm.Physics("edge_reaction", [mode, dim]), is_linear=True)
        u = vfvm.solve(sys, inival=0.0, control=control)
        oc = oracle.Control()
        oc.is_linear = True
        uo, _ = oracle.solve_step(oracle.OracleSystem(g, "edge_reaction", [mode, dim]), np.zeros(g.nnodes), oc)
        assert np.max(np.abs(u.ravel() - uo)) <= SOL_TOL * np.max(np.abs(uo))
        mx.append(float(np.max(u)))
    assert abs(mx[0] - mx[1]) <= 1e-6
    assert abs(mx[0] - mx[2]) <= 1e-3


@pytest.mark.parametrize("assembly", ["edgewise", "cellwise"])
def test_joule_heat_solve_vs_oracle(vfvm, oracle, assembly):
    g = vfvm.simplexgrid(np.linspace(0.0, 3.0, 31), np.linspace(0.0, 1.0, 11))
    params = [1.0, 1.0, 0.5, 1.0, 1.0]
    sys = vfvm.System(g, vfvm.Physics("joule_heat", params), assembly=assembly)
    u = vfvm.solve(sys, inival=0.0, control=vfvm.SolverControl(reltol_linear=1e-10, maxiters_linear=400))
    uo, _ = oracle.solve_step(oracle.OracleSystem(g, "joule_heat", params, assembly=assembly),
                              np.zeros(2 * g.nnodes), oracle.Control())
    assert np.max(np.abs(u.ravel(order="F") - uo)) <= SOL_TOL * np.max(np.abs(uo))
    assert np.max(u[1]) > 100.0  # the Joule heat warmed the conductor
