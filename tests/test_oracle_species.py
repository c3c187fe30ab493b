"""Species restricted to regions in the oracle and the host API (no GPU).

* The oracle reproduces examples/Example230_BoundaryFlux.jl's own check
  (runtests, :205-211): a boundary species solved along the right edge of a 2D
  grid equals the 1D line problem to < 1e-14, for :edgewise and :cellwise.
* The oracle's treatment of the dofs a node does not carry (F += U - Uold, a
  unit diagonal, no coupling to the carried dofs) restates
  src/vfvm_system.jl:1012-1042 and src/vfvm_assemblydata.jl:245-470.
* enable_species / enable_boundary_species / node_species follow
  src/vfvm_system.jl:433-513 (a species is a bulk or a boundary species).
"""
import numpy as np
import pytest

N230 = 20                   # n of Example230.main (an even number)
D1 = DB = 5.0               # d1 = db
KMAX, CMAX = 2.0, 3.0
D2 = K2 = C2 = 1.0


def ex230_oracle(vfvm, oracle, assembly):
    X = np.linspace(0.0, 1.0, N230)
    g1, g2 = vfvm.simplexgrid(X), vfvm.simplexgrid(X, X)
    # the line problem: species 2 as the bulk species of a 1D grid, species 1 nowhere
    o1 = oracle.OracleSystem(g1, "boundary_species", [D2, K2, C2, DB, KMAX, CMAX, 0], assembly=assembly,
                             region_species=np.array([[0], [1]]))
    u1, _ = oracle.solve_step(o1, np.zeros(2 * g1.nnodes), oracle.Control())
    # the 2D problem: species 1 in cell region 1, species 2 on boundary region 2 (x = 1)
    o2 = oracle.OracleSystem(g2, "boundary_species", [D2, K2, C2, DB, KMAX, CMAX, 2], assembly=assembly,
                             region_species=np.array([[1], [0]]),
                             bregion_species=np.array([[0, 0, 0, 0], [0, 1, 0, 0]]))
    u2, _ = oracle.solve_step(o2, np.zeros(2 * g2.nnodes), oracle.Control())
    return g1, g2, u1.reshape(-1, 2).T, u2.reshape(-1, 2).T


def right_edge(g2):
    r = np.flatnonzero(np.abs(g2.coord[0] - 1.0) < 1e-14)
    return r[np.argsort(g2.coord[1, r])]


@pytest.mark.parametrize("assembly", ["edgewise", "cellwise"])
def test_oracle_example230_boundary_equals_line(vfvm, oracle, assembly):
    g1, g2, u1, u2 = ex230_oracle(vfvm, oracle, assembly)
    r = right_edge(g2)
    assert np.linalg.norm(u2[1, r] - u1[1], 2) < 1.0e-14
    # the solution is not trivial, and the dofs the nodes do not carry stay at the start value 0
    assert np.max(u1[1]) > 0.5
    assert np.all(u1[0] == 0.0)
    assert np.all(np.delete(u2[1], r) == 0.0)


def test_oracle_inactive_rows(vfvm, oracle):
    """Dofs a node does not carry: F = U - Uold, a unit diagonal row, and no
    coupling between carried and not-carried dofs in either direction."""
    X = np.linspace(0.0, 1.0, 7)
    g2 = vfvm.simplexgrid(X, X)
    o2 = oracle.OracleSystem(g2, "boundary_species", [D2, K2, C2, DB, KMAX, CMAX, 2],
                             region_species=np.array([[1], [0]]),
                             bregion_species=np.array([[0, 0, 0, 0], [0, 1, 0, 0]]))
    rng = np.random.default_rng(5)
    U = rng.uniform(0.1, 1.0, 2 * g2.nnodes)
    Uold = rng.uniform(0.1, 1.0, 2 * g2.nnodes)
    F, J = o2.assemble(U, Uold)
    carried = np.zeros((2, g2.nnodes), dtype=bool)
    carried[0] = True
    carried[1, right_edge(g2)] = True
    act = carried.ravel(order="F")
    ina = np.flatnonzero(~act)
    assert np.allclose(F[ina], U[ina] - Uold[ina], rtol=0, atol=0)
    Jd = J.toarray()
    assert np.array_equal(Jd[np.ix_(ina, ina)], np.eye(ina.size))
    assert not np.any(Jd[np.ix_(np.flatnonzero(act), ina)])
    assert not np.any(Jd[np.ix_(ina, np.flatnonzero(act))])
    # Dirichlet initialisation sets them to 0 (_initialize_inactive_dof!)
    V = U.copy()
    o2.init_dirichlet(V)
    assert np.all(V[ina] == 0.0) and np.array_equal(V[act], U[act])


def test_oracle_species_conflicts(vfvm, oracle):
    g2 = vfvm.simplexgrid(np.linspace(0, 1, 4), np.linspace(0, 1, 4))
    with pytest.raises(ValueError):  # species 2 both bulk and boundary species
        oracle.OracleSystem(g2, "boundary_species", [1, 1, 1, 1, 1, 1, 2], region_species=np.array([[1], [1]]),
                            bregion_species=np.array([[0, 0, 0, 0], [0, 1, 0, 0]]))
    with pytest.raises(ValueError):  # no species at all
        oracle.OracleSystem(g2, "boundary_species", [1, 1, 1, 1, 1, 1, 2], region_species=np.zeros((2, 1)))


def test_host_species_api(vfvm):
    X = np.linspace(0.0, 1.0, 6)
    g2 = vfvm.simplexgrid(X, X)
    sys = vfvm.System(g2, vfvm.Physics("boundary_species", [1, 1, 1, 1, 1, 1, 2]))
    assert sys.region_species is None and vfvm.node_species(sys).all()
    vfvm.enable_species(sys, 1, [1])
    vfvm.enable_boundary_species(sys, 2, [2])
    ns = vfvm.node_species(sys)
    assert ns[0].all()
    assert np.array_equal(np.flatnonzero(ns[1]), np.sort(right_edge(g2)))
    with pytest.raises(ValueError):
        vfvm.enable_boundary_species(sys, 1, [3])    # already a bulk species
    with pytest.raises(ValueError):
        vfvm.enable_species(sys, 2, [1])             # already a boundary species
    with pytest.raises(ValueError):
        vfvm.enable_species(sys, 3, [1])             # the physics has 2 species
    # species= enables the listed species in every cell region (System(...; species))
    s2 = vfvm.System(g2, vfvm.Physics("rd2", [1, 1, 1]), species=[1])
    assert vfvm.node_species(s2)[0].all() and not vfvm.node_species(s2)[1].any()
    s3 = vfvm.System(g2, vfvm.Physics("rd2", [1, 1, 1]), species=[1, 2])
    assert vfvm.node_species(s3).all()
    with pytest.raises(ValueError):
        vfvm.System(g2, vfvm.Physics("rd2", [1, 1, 1]), unknown_storage="compressed")


def test_host_system_keywords(vfvm):
    """System(...; matrixtype, valuetype, nparams) keywords of the reference."""
    g = vfvm.simplexgrid(np.linspace(0.0, 1.0, 5), np.linspace(0.0, 1.0, 5))
    assert vfvm.System(g, vfvm.Physics("ex430", [0.5]), nparams=1).nparams == 1
    assert vfvm.System(g, vfvm.Physics("nlpoisson"), matrixtype="banded").nparams == 0
    with pytest.raises(ValueError):
        vfvm.System(g, vfvm.Physics("nlpoisson"), nparams=1)
    with pytest.raises(ValueError):
        vfvm.System(g, vfvm.Physics("nlpoisson"), valuetype=np.float32)
    with pytest.raises(ValueError):
        vfvm.System(g, vfvm.Physics("nlpoisson"), matrixtype="dense")
