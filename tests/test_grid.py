import os

import numpy as np
import pytest

from conftest import GOLDEN


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


# --- SimplexGrid text files (.sg)

GOLDEN_SG = os.path.join(GOLDEN, "jittered_square.sg")


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_sg_round_trip(vfvm, tmp_path, dim):
    X = np.linspace(0.0, 1.0, 5) ** 1.5
    g = vfvm.simplexgrid(*([X] * dim))
    p = tmp_path / f"g{dim}.sg"
    vfvm.write_sg(g, p)
    h = vfvm.simplexgrid(str(p))
    for name in ("coord", "cellnodes", "cellregions", "bfacenodes", "bfaceregions"):
        assert np.array_equal(getattr(g, name), getattr(h, name)), name


def test_sg_unstructured_fixture(vfvm, oracle):
    # a Delaunay triangulation of a jittered lattice: the Voronoi volumes add up
    # to the domain's area and no edge factor is negative (Delaunay property)
    g = vfvm.read_sg(GOLDEN_SG)
    assert (g.dim, g.nnodes, g.nbfaces) == (2, 289, 64)
    for reg, (axis, val) in {1: (1, 0.0), 2: (0, 1.0), 3: (1, 1.0), 4: (0, 0.0)}.items():
        nodes = g.bfacenodes[:, g.bfaceregions == reg].ravel()
        assert nodes.size == 32 and np.all(g.coord[axis, nodes] == val)
    osys = oracle.OracleSystem(g, "nlpoisson")
    assert osys.nodevolumes().sum() == pytest.approx(1.0, rel=1e-13)
    _, ef, _ = osys.factors()
    assert np.all(ef > -1e-14)


def test_sg_rejects_malformed(vfvm, tmp_path):
    bad = tmp_path / "bad.sg"
    bad.write_text("SimplexGrid 2.1\nDIMENSION\n2\nNODES\n3 2\n0 0\n1 0\n0 1\nCELLS\n1\n1 2 4 1\nFACES\n0\nEND\n")
    with pytest.raises(ValueError):
        vfvm.read_sg(bad)
    bad.write_text("SimplexGrid 2.1\nDIMENSION\n2\nNODES\n3 2\n0 0\n1 0\n")
    with pytest.raises(ValueError):
        vfvm.read_sg(bad)
    bad.write_text("NotAGrid\n")
    with pytest.raises(ValueError):
        vfvm.read_sg(bad)
