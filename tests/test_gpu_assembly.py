"""GPU assembly parity against the oracle, through the C ABI, for both assembly
kernels (edge-once over node tiles, and node-centric).

* pattern: bit-exact against the entries the reference creates (the oracle's
  _addnz flags, unioned over several states as ExtendableSparse keeps them);
* residual: |F - F_oracle| <= 1e-12 * row scale, row scale = max(|F_i|,
  sum_j |J_ij| |u_j|) -- the magnitude of the terms summed into row i;
* Jacobian: |J - J_oracle| <= 1e-12 * max_j |J_oracle(i, j)| per row.
"""
import numpy as np
import pytest

from gpu_cases import NAMES, case, random_state

pytestmark = pytest.mark.gpu
TOL = 1e-12


def make_pair(vfvm, oracle, c, assembly="edgewise"):
    sys = vfvm.System(c["grid"], vfvm.Physics(c["kind"], c["params"], c["nodedata"]))
    bf = bv = None
    if c["legacy"] is not None:
        bf, bv = c["legacy"]
        for ispec in range(bf.shape[0]):
            for ireg in range(bf.shape[1]):
                if bf[ispec, ireg] == 1e30:
                    vfvm.boundary_dirichlet(sys, ispec + 1, ireg + 1, bv[ispec, ireg])
    osys = oracle.OracleSystem(c["grid"], c["kind"], c["params"], nodedata=c["nodedata"], bfactors=bf, bvalues=bv,
                               assembly=assembly)
    return sys, osys


@pytest.mark.parametrize("kernel", ["tile", "node", "cellwise"])
@pytest.mark.parametrize("name", NAMES)
def test_assembly_parity(vfvm, oracle, name, kernel, monkeypatch):
    # tile: the edge-once kernel over shared-memory node tiles (the default);
    # node: the node-centric kernel (multi-region grids, physics with boundary
    # fluxes; selectable for comparison); cellwise: the default kernel against
    # the oracle's cellwise assembly (the reference's default mode: the same
    # operator summed cell by cell)
    if kernel == "node":
        monkeypatch.setenv("VFVM_ASSEMBLY_KERNEL", "node")
    c = case(vfvm, name)
    sys, osys = make_pair(vfvm, oracle, c, assembly="cellwise" if kernel == "cellwise" else "edgewise")
    rng = np.random.default_rng(42)
    ns = sys.nspec
    # structural pattern in the oracle: union over states (ExtendableSparse keeps entries)
    for _ in range(3):
        osys.assemble(random_state(c, ns, rng).ravel(order="F"), random_state(c, ns, rng).ravel(order="F"),
                      c["t"], c["tstep"], c["embed"], keep_pattern=True)
    U = random_state(c, ns, rng)
    Uold = random_state(c, ns, rng)
    Fo, Jo = osys.assemble(U.ravel(order="F"), Uold.ravel(order="F"), c["t"], c["tstep"], c["embed"], keep_pattern=True)
    F, J = vfvm.evaluate_residual_and_jacobian(sys, U, t=c["t"], tstep=c["tstep"], embed=c["embed"], uold=Uold)
    F = F.ravel(order="F")
    # pattern bit-exact
    Jo.sort_indices()
    assert np.array_equal(J.indptr, Jo.indptr), "row pointers differ"
    assert np.array_equal(J.indices, Jo.indices), "column indices differ"
    # residual
    absJ = abs(Jo)
    rowscale = np.maximum(np.abs(Fo), absJ @ np.abs(U.ravel(order="F")))
    err = np.abs(F - Fo)
    assert np.all(err <= TOL * rowscale + 1e-300), f"max rel residual err {np.max(err / np.maximum(rowscale, 1e-300)):.3e}"
    # Jacobian values on the common pattern
    rowmax = np.maximum.reduceat(np.abs(Jo.data), Jo.indptr[:-1]) if Jo.nnz else np.zeros(0)
    rows = np.repeat(np.arange(Jo.shape[0]), np.diff(Jo.indptr))
    jerr = np.abs(J.data - Jo.data)
    assert np.all(jerr <= TOL * rowmax[rows] + 1e-300), f"max rel jacobian err {np.max(jerr / np.maximum(rowmax[rows], 1e-300)):.3e}"


@pytest.mark.parametrize("name", ["nlpoisson", "ex160", "bipolar", "ex110", "rd2"])
def test_init_dirichlet_parity(vfvm, oracle, name):
    c = case(vfvm, name)
    sys, osys = make_pair(vfvm, oracle, c)
    rng = np.random.default_rng(3)
    U = random_state(c, sys.nspec, rng).ravel(order="F")
    Uo = U.copy()
    osys.init_dirichlet(Uo, c["t"], c["embed"])
    lib = vfvm._lib.load()
    Ug = U.copy()
    assert lib.vfvm_init_dirichlet(sys.ctx, vfvm._lib.ptr(Ug), c["t"], c["embed"]) == 0
    assert np.array_equal(Ug, Uo)


def test_geometry_parity(vfvm, oracle):
    X = np.array([i / 7 for i in range(8)])
    for g in (vfvm.simplexgrid(X), vfvm.simplexgrid(X, X), vfvm.simplexgrid(X, X, X)):
        sys = vfvm.System(g, vfvm.Physics("porous"))
        nv = vfvm.nodevolumes(sys)
        ef, en = vfvm.edgefactors(sys)
        nvo, efo, eno = oracle.OracleSystem(g, "porous").factors()
        assert np.array_equal(en, eno)
        np.testing.assert_allclose(nv, nvo, rtol=1e-13, atol=1e-16)
        np.testing.assert_allclose(ef, efo, rtol=1e-12, atol=1e-14 * np.max(np.abs(efo)))


def test_nan_is_assembly_error(vfvm):
    c = case(vfvm, "nlpoisson")
    sys = vfvm.System(c["grid"], vfvm.Physics("nlpoisson"))
    U = np.full((1, c["grid"].nnodes), 0.5)
    U[0, 5] = np.nan
    with pytest.raises(vfvm.AssemblyError):
        vfvm.evaluate_residual_and_jacobian(sys, U)
