"""The oracle's boundary-edge fluxes, boundary storage and sources, and its
cellwise assembly mode (CPU only).

* cellwise (the reference's default, per-cell factors) and edgewise (factors
  summed per edge) assemble the same operator: residual and Jacobian agree to
  rounding, with the same pattern;
* the Jacobian of the surface-layer physics (bflux, bstorage, bsource,
  breaction) equals central finite differences of the residual, in 2D
  (boundary faces are segments) and 3D (triangles).
"""
import numpy as np
import pytest


def lin(n):
    return np.linspace(0.0, 1.0, n + 1)


@pytest.mark.parametrize("axes,kind,params,ns", [
    ((lin(8), lin(8)), "porous", [], 1),
    ((lin(4), lin(4), lin(4)), "bipolar", [1, 1, 1, 1, 1, 1e3, 0.5], 3),
    ((lin(6), lin(6)), "surface_heat", [1.0, 0.3, 0.5, 2.0, 10.0, 2], 1),
    ((lin(3), lin(3), lin(3)), "surface_heat", [1.0, 0.3, 0.5, 2.0, 10.0, 5], 1),
    ((lin(20),), "ex105", [1e-3], 1),
])
def test_cellwise_equals_edgewise(vfvm, oracle, axes, kind, params, ns):
    g = vfvm.simplexgrid(*axes)
    rng = np.random.default_rng(0)
    U = rng.uniform(0.5, 1.5, size=ns * g.nnodes)
    Uo = rng.uniform(0.5, 1.5, size=ns * g.nnodes)
    Fe, Je = oracle.OracleSystem(g, kind, params).assemble(U, Uo, 0.0, 1e-2, 0.5)
    Fc, Jc = oracle.OracleSystem(g, kind, params, assembly="cellwise").assemble(U, Uo, 0.0, 1e-2, 0.5)
    assert np.array_equal(Je.indptr, Jc.indptr) and np.array_equal(Je.indices, Jc.indices)
    assert np.max(np.abs(Fe - Fc)) <= 1e-14 * np.max(np.abs(Fe))
    assert np.max(np.abs(Je.data - Jc.data)) <= 1e-14 * np.max(np.abs(Je.data))


@pytest.mark.parametrize("axes,breg", [((lin(5), lin(5)), 2), ((lin(3), lin(3), lin(3)), 5)])
def test_surface_heat_jacobian_finite_differences(vfvm, oracle, axes, breg):
    g = vfvm.simplexgrid(*axes)
    params = [1.0, 0.3, 0.5, 2.0, 10.0, breg]
    o = oracle.OracleSystem(g, "surface_heat", params)
    rng = np.random.default_rng(1)
    U = rng.uniform(0.5, 1.5, g.nnodes)
    Uo = rng.uniform(0.5, 1.5, g.nnodes)
    F, J = o.assemble(U, Uo, 0.0, 0.1)
    Jd = J.toarray()
    h = 1e-6
    for k in range(g.nnodes):
        Up, Um = U.copy(), U.copy()
        Up[k] += h
        Um[k] -= h
        fd = (o.assemble(Up, Uo, 0.0, 0.1)[0] - o.assemble(Um, Uo, 0.0, 0.1)[0]) / (2 * h)
        assert np.max(np.abs(fd - Jd[:, k])) <= 1e-6 * np.max(np.abs(Jd))
    # the boundary terms are active: switching them off changes the residual
    F0, _ = oracle.OracleSystem(g, "surface_heat", [1.0, 0.0, 0.0, 0.0, 0.0, breg]).assemble(U, Uo, 0.0, 0.1)
    assert np.max(np.abs(F - F0)) > 0.1
