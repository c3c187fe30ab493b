"""Oracle unit tests restating the reference's unit tests (test/test010, 020, 080, 120)."""
import ctypes
import os

import numpy as np
import pytest

from conftest import GOLDEN


def test_bernoulli_kat(oracle):
    # test/test010_bernoulli.jl: max abs error < 1e-14 against high precision
    kat = np.load(os.path.join(GOLDEN, "bernoulli_kat.npz"))
    x = np.ascontiguousarray(kat["x"])
    bp = np.zeros_like(x)
    bm = np.zeros_like(x)
    L = oracle.lib()
    P = ctypes.POINTER(ctypes.c_double)
    L.oracle_fbernoulli_pm(x.ctypes.data_as(P), bp.ctypes.data_as(P), bm.ctypes.data_as(P), x.size)
    assert np.max(np.abs(bp - kat["bp"])) < 1e-14
    assert np.max(np.abs(bm - kat["bm"])) < 1e-14


def test_formfactors_triangle_vs_bface(oracle):
    # test/test020_formfactors.jl: 2D cell factors == 3D bface factors of the same triangle
    rng = np.random.default_rng(12345)
    L = oracle.lib()
    P = ctypes.POINTER
    nodes = np.array([0, 1, 2], dtype=np.int32)
    for _ in range(100):
        c2 = np.round(rng.uniform(-10, 10, size=(3, 2)), 2)  # rand(-10:0.01:10, 2, 3), node-major
        c3 = np.hstack([c2, np.zeros((3, 1))])
        n2, e2, n3, e3 = (np.zeros(3) for _ in range(4))
        c2 = np.ascontiguousarray(c2); c3 = np.ascontiguousarray(c3)
        L.oracle_cellfactors(2, c2.ctypes.data_as(P(ctypes.c_double)), nodes.ctypes.data_as(P(ctypes.c_int)),
                             n2.ctypes.data_as(P(ctypes.c_double)), e2.ctypes.data_as(P(ctypes.c_double)))
        L.oracle_bfacefactors_raw(3, c3.ctypes.data_as(P(ctypes.c_double)), nodes.ctypes.data_as(P(ctypes.c_int)),
                                  n3.ctypes.data_as(P(ctypes.c_double)), e3.ctypes.data_as(P(ctypes.c_double)))
        np.testing.assert_allclose(n3, n2, rtol=1e-7)
        np.testing.assert_allclose(e3, e2, rtol=1e-7)


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_nodevolumes_sum(oracle, vfvm, dim):
    # test/test120_norms.jl:103-108,129: sum(nodevolumes) == 1 on the unit cube
    X = np.array([i / 10 for i in range(11)])
    g = vfvm.simplexgrid(*([X] * dim))
    s = oracle.OracleSystem(g, "porous")
    assert s.nodevolumes().sum() == pytest.approx(1.0, rel=1e-13)


def test_checkdelaunay(oracle, vfvm):
    # test/test080_checkdelaunay.jl: uniform grid has no negative edge factors, a jittered one has some
    X = np.array([i / 10 for i in range(101)])
    g = vfvm.simplexgrid(X, X)
    _, ef, _ = oracle.OracleSystem(g, "porous").factors()
    assert np.sum(ef < -1e-12) == 0
    rng = np.random.default_rng(1)
    g.coord += 0.01 * (rng.random(g.coord.shape) - 0.5)
    _, ef, _ = oracle.OracleSystem(g, "porous").factors()
    assert np.sum(ef < 0) > 0


def test_oracle_mass_matrix_storage_u(vfvm, oracle):
    """mass_matrix for storage u (porous medium): the node volumes on the diagonal."""
    X = np.linspace(0.0, 1.0, 9)
    g = vfvm.simplexgrid(X, X)
    o = oracle.OracleSystem(g, "porous")
    M = o.mass_matrix()
    assert np.allclose(M.toarray(), np.diag(o.nodevolumes()), rtol=1e-15, atol=0)
