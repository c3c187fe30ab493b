"""Write ``tests/golden/jittered_square.sg``: an unstructured triangulation of
the unit square in the SimplexGrid text format, for the ``.sg`` reader tests and
solves on a non-tensor grid.

Points: a 17 x 17 lattice whose interior points are moved by up to 0.15 of the
spacing (numpy PCG64, seed 7); boundary points stay on the sides.  Cells: the
Delaunay triangulation of the points (scipy/Qhull), every triangle oriented
counter-clockwise.  Boundary faces: consecutive boundary points of each side,
with the ``simplexgrid`` region numbers (1 south, 2 east, 3 north, 4 west).

    python tests/golden/make_unstructured_grid.py
"""
import os
import sys

import numpy as np
from scipy.spatial import Delaunay

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def jittered_square(n=17, jitter=0.15, seed=7):
    import __graft_entry__
    vfvm = __graft_entry__.load_package()
    h = 1.0 / (n - 1)
    x = np.linspace(0.0, 1.0, n)
    X, Y = np.meshgrid(x, x)
    pts = np.stack([X.ravel(), Y.ravel()], axis=1)
    inner = (pts[:, 0] > 0) & (pts[:, 0] < 1) & (pts[:, 1] > 0) & (pts[:, 1] < 1)
    rng = np.random.default_rng(seed)
    pts[inner] += jitter * h * (2.0 * rng.random((int(inner.sum()), 2)) - 1.0)
    cells = Delaunay(pts).simplices.copy()
    a, b, c = pts[cells[:, 0]], pts[cells[:, 1]], pts[cells[:, 2]]
    det = (b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0])
    cells[det < 0, 1], cells[det < 0, 2] = cells[det < 0, 2], cells[det < 0, 1].copy()
    faces, regions = [], []
    for region, (axis, value, along) in {1: (1, 0.0, 0), 2: (0, 1.0, 1), 3: (1, 1.0, 0), 4: (0, 0.0, 1)}.items():
        side = np.flatnonzero(pts[:, axis] == value)
        side = side[np.argsort(pts[side, along])]
        for i in range(side.size - 1):
            faces.append((side[i], side[i + 1]))
            regions.append(region)
    return vfvm.Grid(pts.T, cells.T, np.ones(len(cells), dtype=np.int32), np.array(faces).T, np.array(regions))


if __name__ == "__main__":
    import __graft_entry__
    vfvm = __graft_entry__.load_package()
    vfvm.write_sg(jittered_square(), os.path.join(HERE, "jittered_square.sg"))
