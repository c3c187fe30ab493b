"""Edge reactions in the oracle (no GPU).

examples/DevEx002_EdgeReaction.jl's own check (runtests, :181-205, case
:compare_max): the unit source given as a node reaction, as the edge reaction
-meas(edge)^2/(2 dim) and as -(phi_K - phi_L)^2/2 gives the same solution
maximum (atol 1e-6 and 1e-3).  The example's runtests loops over dim = 1:3 but
passes no dim (so it runs its Triangulate grid three times); here the three
dimensions run on tensor-product simplex grids with its spacing 0.25.
"""
import numpy as np
import pytest


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_oracle_devex002_compare_max(vfvm, oracle, dim):
    X = np.arange(0.0, 1.0 + 1e-12, 0.25)
    g = vfvm.simplexgrid(*([X] * dim))
    c = oracle.Control()
    c.is_linear = True
    mx = []
    for mode in (0, 1, 2):
        u, _ = oracle.solve_step(oracle.OracleSystem(g, "edge_reaction", [mode, dim]), np.zeros(g.nnodes), c)
        mx.append(float(np.max(u)))
    assert mx[0] > 0.01
    assert abs(mx[0] - mx[1]) <= 1e-6
    assert abs(mx[0] - mx[2]) <= 1e-3


def test_oracle_edgereaction_residual_and_sign_placement(vfvm, oracle):
    """The residual of an edge reaction goes to both end nodes with the same
    sign; the Jacobian takes the entries src/vfvm_assembly.jl:213-229 places:
    the diagonal blocks are the derivative of the residual, the coupling
    blocks carry the opposite sign of it."""
    g = vfvm.simplexgrid(np.array([0.0, 1.0]))  # one edge, nodes 0 and 1
    o = oracle.OracleSystem(g, "joule_heat", [1.0, 1.0, 0.5, 1.0, 1.0])
    u = np.array([0.3, 0.2, 0.9, 0.6])  # (phi, T) at node 0, then node 1
    F, J = o.assemble(u)
    Jd = J.toarray()
    eps = 1e-7
    Jfd = np.zeros((4, 4))
    for k in range(4):
        up, um = u.copy(), u.copy()
        up[k] += eps
        um[k] -= eps
        Jfd[:, k] = (o.assemble(up)[0] - o.assemble(um)[0]) / (2 * eps)
    # the T rows (1, 3) hold the edge reaction's partials in the phi columns (0, 2)
    assert np.allclose(Jd[1, 0], Jfd[1, 0], rtol=1e-6) and np.allclose(Jd[3, 2], Jfd[3, 2], rtol=1e-6)
    assert np.allclose(Jd[1, 2], -Jfd[1, 2], rtol=1e-6) and np.allclose(Jd[3, 0], -Jfd[3, 0], rtol=1e-6)
    assert abs(Jfd[1, 2]) > 0.1
