import numpy as np
import pytest


@pytest.mark.parametrize("dim,ncells_per_box", [(1, 1), (2, 2), (3, 6)])
def test_simplexgrid_counts(vfvm, dim, ncells_per_box):
    X = np.linspace(0, 1, 5)
    g = vfvm.simplexgrid(*([X] * dim))
    assert g.nnodes == 5 ** dim
    assert g.ncells == ncells_per_box * 4 ** dim
    assert g.cellnodes.min() == 0 and g.cellnodes.max() == g.nnodes - 1
    assert g.bfaceregions.max() == 2 * dim


def test_simplexgrid_regions_2d(vfvm):
    X = np.linspace(0, 1, 4)
    g = vfvm.simplexgrid(X, X)
    for reg, (axis, val) in {1: (1, 0.0), 2: (0, 1.0), 3: (1, 1.0), 4: (0, 0.0)}.items():
        nodes = g.bfacenodes[:, g.bfaceregions == reg].ravel()
        assert np.all(g.coord[axis, nodes] == val)


def test_simplexgrid_regions_3d(vfvm):
    X = np.linspace(0, 1, 4)
    g = vfvm.simplexgrid(X, X, X)
    for reg, (axis, val) in {1: (1, 0.0), 2: (0, 1.0), 3: (1, 1.0), 4: (0, 0.0), 5: (2, 0.0), 6: (2, 1.0)}.items():
        nodes = g.bfacenodes[:, g.bfaceregions == reg].ravel()
        assert np.all(g.coord[axis, nodes] == val)


def test_tet_volumes_positive(vfvm):
    X = np.linspace(0, 1, 3)
    g = vfvm.simplexgrid(X, X, X)
    c = g.coord
    v = []
    for k in range(g.ncells):
        n = g.cellnodes[:, k]
        a, b, d = c[:, n[1]] - c[:, n[0]], c[:, n[2]] - c[:, n[0]], c[:, n[3]] - c[:, n[0]]
        v.append(abs(np.dot(a, np.cross(b, d))) / 6)
    assert sum(v) == pytest.approx(1.0)
    assert min(v) > 0
