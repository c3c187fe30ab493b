"""Species restricted to regions on the GPU, through the C ABI, against the oracle.

enable_species! / enable_boundary_species! (src/vfvm_system.jl:433-513) with
the dense unknown layout: each term assembles the rows and columns of its
region's (cell terms) or node's (boundary terms) species
(src/vfvm_assemblydata.jl:245-470); the dofs a node does not carry get
F += U - Uold and a unit diagonal (src/vfvm_system.jl:1012-1026) and start at
0 (:1030-1042).

* assembly: pattern bit-exact, residual and Jacobian within 1e-12 of the row
  scale (the tolerances of the unrestricted assembly parity test), edgewise
  and cellwise;
* examples/Example230_BoundaryFlux.jl on the GPU: the boundary species along
  x = 1 of the 2D grid equals the GPU's 1D line solve.  The reference checks
  < 1e-14 with a direct solver; here each Newton step solves with BiCGStab to
  a relative 1e-10, so the two solves stop at different iterates within the
  Newton tolerance: the bound is 1e-11 (the solution is about 1.5);
* solves (stationary two-region reaction-diffusion, transient two-species
  steps with device step control) against the oracle within 1e-8 relative.
"""
import numpy as np
import pytest

from gpu_cases import lin

pytestmark = pytest.mark.gpu
TOL = 1e-12
SOL_TOL = 1e-8
EX230 = dict(d=1.0, k=1.0, c=1.0, db=5.0, kmax=2.0, cmax=3.0)  # Example230.main defaults (d2 = k2 = c2 = 1)


def ex230_params(breg):
    e = EX230
    return [e["d"], e["k"], e["c"], e["db"], e["kmax"], e["cmax"], breg]


def two_regions(vfvm, g):
    """The same grid with the cells right of x = 1/2 in cell region 2."""
    cx = g.coord[0, g.cellnodes].mean(axis=0)
    return vfvm.Grid(g.coord, g.cellnodes, np.where(cx > 0.5, 2, 1), g.bfacenodes, g.bfaceregions)


def species_case(vfvm, name):
    """(grid, kind, params, region_species, bregion_species, tstep)"""
    if name == "ex230":
        g = vfvm.simplexgrid(lin(8), lin(8))
        return g, "boundary_species", ex230_params(2), np.array([[1], [0]]), np.array([[0, 0, 0, 0], [0, 1, 0, 0]]), np.inf
    if name == "ex230_line":
        g = vfvm.simplexgrid(lin(12))
        return g, "boundary_species", ex230_params(0), np.array([[0], [1]]), np.zeros((2, 2), dtype=int), np.inf
    if name == "rd2_two_regions":
        g = two_regions(vfvm, vfvm.simplexgrid(lin(8), lin(8)))
        return g, "rd2", [0.5, 2.0, 3.0], np.array([[1, 1], [0, 1]]), np.zeros((2, 4), dtype=int), np.inf
    if name == "ex110_two_regions":
        g = two_regions(vfvm, vfvm.simplexgrid(lin(16)))
        return g, "ex110", [0.5, 0.5], np.array([[1, 1], [0, 1]]), np.zeros((2, 2), dtype=int), 1e-2
    if name == "ex115":  # Example115: boundary species C on the catalytic end (region 1), B = 0 at the other
        g = vfvm.simplexgrid(lin(10))
        bs = np.zeros((3, 2), dtype=int)
        bs[2, 0] = 1
        return g, "ex115", [1.0, 1.0e-2, 100.0, 1.0, 0.1, 1.0, 0.01, 1], np.array([[1], [1], [0]]), bs, 1e-2
    if name == "ex220":  # Example220: boundary species 3 on region 2 of a 2D grid
        g = vfvm.simplexgrid(lin(8), lin(8))
        bs = np.zeros((3, 4), dtype=int)
        bs[2, 1] = 1
        return g, "ex220", [1.0, 1.0e-2], np.array([[1], [1], [0]]), bs, 1e-2
    raise KeyError(name)


NAMES = ["ex230", "ex230_line", "rd2_two_regions", "ex110_two_regions", "ex115", "ex220"]


def make_pair(vfvm, oracle, name, assembly="edgewise", unknown_storage="dense"):
    g, kind, params, rs, bs, tstep = species_case(vfvm, name)
    sys = vfvm.System(g, vfvm.Physics(kind, params), assembly=assembly, unknown_storage=unknown_storage)
    for i in range(rs.shape[0]):
        regs = [r + 1 for r in range(rs.shape[1]) if rs[i, r]]
        if regs:
            vfvm.enable_species(sys, i + 1, regs)
        bregs = [r + 1 for r in range(bs.shape[1]) if bs[i, r]]
        if bregs:
            vfvm.enable_boundary_species(sys, i + 1, bregs)
    osys = oracle.OracleSystem(g, kind, params, assembly=assembly, region_species=rs, bregion_species=bs)
    return sys, osys, tstep


@pytest.mark.parametrize("assembly", ["edgewise", "cellwise"])
@pytest.mark.parametrize("name", NAMES)
def test_species_assembly_parity(vfvm, oracle, name, assembly):
    sys, osys, tstep = make_pair(vfvm, oracle, name, assembly)
    assert sys.info()["multiregion"]  # restricted species take the node-centric multi-item kernel
    rng = np.random.default_rng(11)
    n = sys.ndofs
    for _ in range(3):  # structural pattern: union over states (ExtendableSparse keeps entries)
        osys.assemble(rng.uniform(0.2, 1.2, n), rng.uniform(0.2, 1.2, n), 0.0, tstep, 0.0, keep_pattern=True)
    U = rng.uniform(0.2, 1.2, n)
    Uold = rng.uniform(0.2, 1.2, n)
    Fo, Jo = osys.assemble(U, Uold, 0.0, tstep, 0.0, keep_pattern=True)
    F, J = vfvm.evaluate_residual_and_jacobian(sys, U, tstep=tstep, uold=Uold)
    F = F.ravel(order="F")
    Jo.sort_indices()
    assert np.array_equal(J.indptr, Jo.indptr), "row pointers differ"
    assert np.array_equal(J.indices, Jo.indices), "column indices differ"
    rowscale = np.maximum(np.abs(Fo), abs(Jo) @ np.abs(U))
    assert np.all(np.abs(F - Fo) <= TOL * rowscale + 1e-300)
    rowmax = np.maximum.reduceat(np.abs(Jo.data), Jo.indptr[:-1])
    rows = np.repeat(np.arange(Jo.shape[0]), np.diff(Jo.indptr))
    assert np.all(np.abs(J.data - Jo.data) <= TOL * rowmax[rows] + 1e-300)


@pytest.mark.parametrize("name", NAMES)
def test_species_init_dirichlet(vfvm, oracle, name):
    sys, osys, _ = make_pair(vfvm, oracle, name)
    U = np.random.default_rng(4).uniform(0.2, 1.2, sys.ndofs)
    Uo = U.copy()
    osys.init_dirichlet(Uo)
    Ug = U.copy()
    lib = vfvm._lib.load()
    assert lib.vfvm_init_dirichlet(sys.ctx, vfvm._lib.ptr(Ug), 0.0, 0.0) == 0
    assert np.array_equal(Ug, Uo)
    assert np.all(Ug[~vfvm.node_species(sys).ravel(order="F")] == 0.0)


def right_edge(g):
    r = np.flatnonzero(np.abs(g.coord[0] - 1.0) < 1e-14)
    return r[np.argsort(g.coord[1, r])]


@pytest.mark.parametrize("assembly", ["edgewise", "cellwise"])
@pytest.mark.parametrize("storage", ["dense", "sparse"])
def test_example230_gpu_boundary_equals_line(vfvm, oracle, storage, assembly):
    """examples/Example230_BoundaryFlux.jl:186-211 on the GPU (n = 20)."""
    X = np.linspace(0.0, 1.0, 20)
    g1, g2 = vfvm.simplexgrid(X), vfvm.simplexgrid(X, X)
    control = vfvm.SolverControl(reltol_linear=1e-10, maxiters_linear=400)
    s1 = vfvm.System(g1, vfvm.Physics("boundary_species", ex230_params(0)), assembly=assembly,
                     unknown_storage=storage)
    vfvm.enable_species(s1, 2, [1])
    u1 = vfvm.solve(s1, inival=0.0, control=control)
    s2 = vfvm.System(g2, vfvm.Physics("boundary_species", ex230_params(2)), assembly=assembly,
                     unknown_storage=storage)
    vfvm.enable_species(s2, 1, [1])
    vfvm.enable_boundary_species(s2, 2, [2])
    u2 = vfvm.solve(s2, inival=0.0, control=control)
    r = right_edge(g2)
    assert np.linalg.norm(u2[1, r] - u1[1], 2) < 1e-11
    assert np.max(u1[1]) > 1.0
    # against the oracle's (direct-solver) 2D solution
    o2 = oracle.OracleSystem(g2, "boundary_species", ex230_params(2), assembly=assembly,
                             region_species=np.array([[1], [0]]),
                             bregion_species=np.array([[0, 0, 0, 0], [0, 1, 0, 0]]))
    uo, _ = oracle.solve_step(o2, np.zeros(2 * g2.nnodes), oracle.Control())
    uo = uo.reshape(-1, 2).T
    assert np.max(np.abs(u2 - uo)) <= SOL_TOL * np.max(np.abs(uo))
    # dofs a node does not carry: 0 (dense: Newton holds them at the start value 0)
    assert np.all(np.delete(u2[1], r) == 0.0) and np.all(u1[0] == 0.0)


def test_sparse_storage_system(vfvm, oracle):
    """unknown_storage = :sparse: the residual and Jacobian of the carried dofs
    only, in the sparse dof order (node-major, species ascending)."""
    sys, osys, tstep = make_pair(vfvm, oracle, "rd2_two_regions", unknown_storage="sparse")
    rng = np.random.default_rng(2)
    U = rng.uniform(0.2, 1.2, sys.ndofs)
    F, J = vfvm.evaluate_residual_and_jacobian(sys, U)
    Fo, Jo = osys.assemble(U, U, 0.0, tstep, 0.0)
    act = np.flatnonzero(vfvm.node_species(sys).ravel(order="F"))
    assert F.shape == (act.size,) and J.shape == (act.size, act.size)
    assert np.allclose(F, Fo[act], rtol=1e-12, atol=1e-14)
    assert np.allclose(J.toarray(), Jo.toarray()[np.ix_(act, act)], rtol=1e-12, atol=1e-14)


def test_two_region_species_solve_vs_oracle(vfvm, oracle):
    sys, osys, _ = make_pair(vfvm, oracle, "rd2_two_regions")
    U = vfvm.solve(sys, inival=0.5, control=vfvm.SolverControl(reltol_linear=1e-8, maxiters_linear=400))
    uo, _ = oracle.solve_step(osys, np.full(sys.ndofs, 0.5), oracle.Control())
    assert np.max(np.abs(U.ravel(order="F") - uo)) <= SOL_TOL * np.max(np.abs(uo))
    # species 2 only right of x = 1/2; elsewhere the unit rows F = U - Uold take
    # U from the start value 0 back to Uold = inival = 0.5
    ns = vfvm.node_species(sys)
    assert np.max(np.abs(U[~ns] - 0.5)) <= 1e-10


@pytest.mark.parametrize("step_control", ["device", "host"])
def test_two_region_species_transient_vs_oracle(vfvm, oracle, step_control):
    sys, osys, _ = make_pair(vfvm, oracle, "ex110_two_regions")
    vfvm.boundary_dirichlet(sys, 1, 1, 1.0)
    vfvm.boundary_dirichlet(sys, 1, 2, 0.0)
    bf = np.zeros((2, 2)); bv = np.zeros((2, 2))
    bf[0, :] = 1e30; bv[0, 0] = 1.0
    g, kind, params, rs, bs, _ = species_case(vfvm, "ex110_two_regions")
    osys = oracle.OracleSystem(g, kind, params, bfactors=bf, bvalues=bv, region_species=rs, bregion_species=bs)
    u0 = np.full(sys.ndofs, 0.3)
    control = vfvm.fixed_timesteps(vfvm.SolverControl(reltol_linear=1e-8, maxiters_linear=400,
                                                      step_control=step_control), 0.05)
    tsol = vfvm.solve(sys, inival=u0.reshape(sys.nspec, -1, order="F"), times=[0.0, 0.25], control=control)
    _, osols, _ = oracle.solve_transient(osys, u0, [0.0, 0.25], oracle.fixed_timesteps(oracle.Control(), 0.05))
    assert len(tsol.u) == len(osols)
    ref = np.asarray(osols[-1])
    assert np.max(np.abs(tsol.u[-1].ravel(order="F") - ref)) <= SOL_TOL * np.max(np.abs(ref))


def test_species_batch_rejected(vfvm):
    g = two_regions(vfvm, vfvm.simplexgrid(lin(8), lin(8)))
    systems = []
    for _ in range(2):
        s = vfvm.System(g, vfvm.Physics("rd2", [0.5, 2.0, 3.0]))
        vfvm.enable_species(s, 1, [1, 2])
        vfvm.enable_species(s, 2, [2])
        systems.append(s)
    with pytest.raises(ValueError):
        vfvm.BatchSolver(systems)
