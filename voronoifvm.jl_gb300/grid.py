"""Tensor-product simplex grids and the derived tables the assembler consumes.

The reference takes its grids from ExtendableGrids.jl (an unvendored dependency,
compat ``ExtendableGrids = "1.11"`` in ``Project.toml``).  Its call sites are
``simplexgrid(X)``, ``simplexgrid(X, Y)`` and ``simplexgrid(X, Y, Z)`` (for example
``examples/Example105_NonlinearPoisson1D.jl:34``,
``examples/Example201_Laplace2D.jl:26``, ``examples/Example301_Laplace3D.jl:30``)
and the grid components ``Coordinates``, ``CellNodes``, ``CellRegions``,
``BFaceNodes`` and ``BFaceRegions`` read in ``src/vfvm_system.jl:690-755``.

This module restates the published ``simplexgrid`` convention:

* nodes are numbered with x fastest, then y, then z;
* 1D: cells ``(i, i+1)``, boundary points region 1 (left) and 2 (right);
* 2D: every rectangle is cut along its lower-left/upper-right diagonal into two
  triangles; boundary regions 1 = south (y min), 2 = east (x max),
  3 = north (y max), 4 = west (x min);
* 3D: every brick is cut into the six Kuhn tetrahedra that share its main
  diagonal; boundary regions 1-4 as in 2D for the side faces, 5 = bottom
  (z min), 6 = top (z max); boundary quads are cut along the diagonal that
  matches the tetrahedral faces.

On uniform rectangular grids the Voronoi weight of every cut diagonal is zero
up to rounding, so the discrete operators do not depend on the cut direction.
The golden values of the reference's examples pin these conventions (see the
oracle tests).

All index arrays here are 0-based int32; coordinates are float64 with shape
``(dim, nnodes)`` (column-major like the reference's ``coord[idim, inode]``).
"""
from __future__ import annotations

import os

import numpy as np

__all__ = ["Grid", "simplexgrid", "circular_symmetric", "spherical_symmetric"]

# CoordinateSystem of an ExtendableGrids grid: which body the grid's coordinates
# describe, and so which form factors the assembly uses
# (src/vfvm_formfactors.jl:12-332)
COORD_SYSTEMS = ("cartesian", "polar1d", "spherical1d", "cylindrical2d")


class Grid:
    """Simplex grid: coordinates, cells, boundary faces and their regions."""

    def __init__(self, coord, cellnodes, cellregions, bfacenodes, bfaceregions):
        self.coord = np.ascontiguousarray(coord, dtype=np.float64)
        self.cellnodes = np.ascontiguousarray(cellnodes, dtype=np.int32)
        self.cellregions = np.ascontiguousarray(cellregions, dtype=np.int32)
        self.bfacenodes = np.ascontiguousarray(bfacenodes, dtype=np.int32)
        self.bfaceregions = np.ascontiguousarray(bfaceregions, dtype=np.int32)
        self.dim = self.coord.shape[0]
        self.coordsystem = "cartesian"
        if self.cellnodes.shape[0] != self.dim + 1:
            raise ValueError("cellnodes must have dim+1 rows")
        if self.bfacenodes.shape[0] != self.dim:
            raise ValueError("bfacenodes must have dim rows")

    @property
    def nnodes(self) -> int:
        return self.coord.shape[1]

    @property
    def ncells(self) -> int:
        return self.cellnodes.shape[1]

    @property
    def nbfaces(self) -> int:
        return self.bfacenodes.shape[1]

    @property
    def num_cellregions(self) -> int:
        return int(self.cellregions.max()) if self.ncells else 0

    @property
    def num_bfaceregions(self) -> int:
        return int(self.bfaceregions.max()) if self.nbfaces else 0

    def edges(self) -> np.ndarray:
        """Unique cell edges as a ``(2, nedges)`` array, oriented low -> high node
        index and sorted lexicographically (the orientation convention used by
        this package for flux evaluation)."""
        d = self.dim
        pairs = []
        for a in range(d + 1):
            for b in range(a + 1, d + 1):
                pairs.append(np.stack([self.cellnodes[a], self.cellnodes[b]]))
        e = np.concatenate(pairs, axis=1)
        e = np.sort(e, axis=0)
        key = e[0].astype(np.int64) * self.nnodes + e[1]
        key = np.unique(key)
        return np.stack([key // self.nnodes, key % self.nnodes]).astype(np.int32)

    def __repr__(self):
        cs = "" if self.coordsystem == "cartesian" else f", coordsystem={self.coordsystem}"
        return (f"Grid(dim={self.dim}, nnodes={self.nnodes}, ncells={self.ncells}, "
                f"nbfaces={self.nbfaces}{cs})")


# --- SimplexGrid text files (ExtendableGrids' ``.sg`` format, e.g. assets/rz2d.sg)
#
#   SimplexGrid 2.1            version line (2.0 and 2.1 share this layout)
#   # ...                      comment lines anywhere
#   DIMENSION  d
#   NODES      nnodes d        then nnodes * d coordinates, node after node
#   CELLS      ncells          then per cell: d+1 node numbers (1-based), region
#   FACES      nbfaces         then per boundary face: d node numbers (1-based), region
#   END

SG_VERSION = "2.1"


def read_sg(path) -> Grid:
    """Read a SimplexGrid text file into a Grid (node numbers become 0-based)."""
    with open(path) as f:
        lines = [ln.split("#", 1)[0].strip() for ln in f]
    lines = [ln for ln in lines if ln]
    if not lines or not lines[0].startswith("SimplexGrid"):
        raise ValueError(f"{path}: not a SimplexGrid file")
    version = lines[0].split()[1] if len(lines[0].split()) > 1 else ""
    if not version.startswith("2."):
        raise ValueError(f"{path}: unsupported SimplexGrid version {version!r}")
    tok = " ".join(lines[1:]).split()
    pos = 0

    def take(n, conv):
        nonlocal pos
        if pos + n > len(tok):
            raise ValueError(f"{path}: truncated")
        out = [conv(t) for t in tok[pos:pos + n]]
        pos += n
        return out

    def expect(key):
        if take(1, str)[0] != key:
            raise ValueError(f"{path}: expected {key} at token {pos - 1}")

    expect("DIMENSION")
    dim = take(1, int)[0]
    if dim not in (1, 2, 3):
        raise ValueError(f"{path}: dimension {dim}")
    expect("NODES")
    nn, d2 = take(2, int)
    if d2 != dim:
        raise ValueError(f"{path}: node dimension {d2} != {dim}")
    coord = np.array(take(nn * dim, float)).reshape(nn, dim).T
    expect("CELLS")
    nc = take(1, int)[0]
    cells = np.array(take(nc * (dim + 2), int), dtype=np.int64).reshape(nc, dim + 2)
    expect("FACES")
    nf = take(1, int)[0]
    faces = np.array(take(nf * (dim + 1), int), dtype=np.int64).reshape(nf, dim + 1)
    expect("END")
    for a in (cells[:, :dim + 1], faces[:, :dim]):
        if a.size and (a.min() < 1 or a.max() > nn):
            raise ValueError(f"{path}: node number out of range")
    return Grid(coord, (cells[:, :dim + 1] - 1).T, cells[:, dim + 1], (faces[:, :dim] - 1).T, faces[:, dim])


def write_sg(grid: Grid, path):
    """Write a Grid as a SimplexGrid 2.1 text file (node numbers 1-based)."""
    d = grid.dim
    with open(path, "w") as f:
        f.write(f"SimplexGrid {SG_VERSION}\n#written by voronoifvm.jl_gb300\nDIMENSION\n{d}\n")
        f.write(f"NODES\n{grid.nnodes} {d}\n")
        for k in range(grid.nnodes):
            f.write(" ".join(repr(float(x)) for x in grid.coord[:, k]) + "\n")
        f.write(f"CELLS\n{grid.ncells}\n")
        for c in range(grid.ncells):
            f.write(" ".join(str(int(i) + 1) for i in grid.cellnodes[:, c]) + f" {int(grid.cellregions[c])}\n")
        f.write(f"FACES\n{grid.nbfaces}\n")
        for b in range(grid.nbfaces):
            f.write(" ".join(str(int(i) + 1) for i in grid.bfacenodes[:, b]) + f" {int(grid.bfaceregions[b])}\n")
        f.write("END\n")


def _as_coords(X):
    X = np.asarray(X, dtype=np.float64).ravel()
    if X.size < 2 or np.any(np.diff(X) <= 0):
        raise ValueError("coordinate vectors must be strictly increasing with >= 2 entries")
    return X


def _mask(grid: Grid, nodes: np.ndarray, maskmin, maskmax, tol: float) -> np.ndarray:
    lo = np.asarray(maskmin, dtype=np.float64).reshape(-1, 1) - tol
    hi = np.asarray(maskmax, dtype=np.float64).reshape(-1, 1) + tol
    inside = np.ones(nodes.shape[1], dtype=bool)
    for v in range(nodes.shape[0]):
        x = grid.coord[:, nodes[v]]
        inside &= np.all((x >= lo) & (x <= hi), axis=0)
    return inside


def circular_symmetric(grid: Grid) -> Grid:
    """circular_symmetric!(grid) (ExtendableGrids; used in
    examples/Example203_CoordinateSystems.jl): a 1D grid's coordinate is the
    radius of a disk or ring (Polar1D), a 2D grid's coordinates are (r, z) of a
    cylinder (Cylindrical2D)."""
    if grid.dim == 1:
        grid.coordsystem = "polar1d"
    elif grid.dim == 2:
        grid.coordsystem = "cylindrical2d"
    else:
        raise ValueError("circular symmetry needs a 1D or 2D grid")
    return grid


def spherical_symmetric(grid: Grid) -> Grid:
    """spherical_symmetric!(grid) (ExtendableGrids): a 1D grid's coordinate is
    the radius of a ball or spherical shell (Spherical1D)."""
    if grid.dim != 1:
        raise ValueError("spherical symmetry needs a 1D grid")
    grid.coordsystem = "spherical1d"
    return grid


def cellmask(grid: Grid, maskmin, maskmax, ireg: int, tol: float = 1e-10) -> Grid:
    """cellmask!(grid, maskmin, maskmax, ireg) (ExtendableGrids): the cells whose
    nodes all lie in the box [maskmin, maskmax] (widened by tol) get region ireg."""
    grid.cellregions[_mask(grid, grid.cellnodes, maskmin, maskmax, tol)] = ireg
    return grid


def bfacemask(grid: Grid, maskmin, maskmax, ireg: int, tol: float = 1e-10) -> Grid:
    """bfacemask!(grid, maskmin, maskmax, ireg) (ExtendableGrids): the boundary
    faces whose nodes all lie in the box [maskmin, maskmax] (widened by tol) get
    boundary region ireg."""
    grid.bfaceregions[_mask(grid, grid.bfacenodes, maskmin, maskmax, tol)] = ireg
    return grid


def simplexgrid(*axes) -> Grid:
    """Create a 1D, 2D or 3D simplex grid from tensor-product coordinate vectors,
    or read one from a SimplexGrid text file (``simplexgrid(path)``, as in
    ``examples/Example203_CoordinateSystems.jl:105``)."""
    if len(axes) == 1 and isinstance(axes[0], (str, os.PathLike)):
        return read_sg(axes[0])
    if len(axes) == 1:
        return _grid1d(_as_coords(axes[0]))
    if len(axes) == 2:
        return _grid2d(_as_coords(axes[0]), _as_coords(axes[1]))
    if len(axes) == 3:
        return _grid3d(*(_as_coords(a) for a in axes))
    raise ValueError("simplexgrid takes 1, 2 or 3 coordinate vectors")


def _grid1d(X):
    n = X.size
    coord = X.reshape(1, n)
    i = np.arange(n - 1, dtype=np.int32)
    cellnodes = np.stack([i, i + 1])
    cellregions = np.ones(n - 1, dtype=np.int32)
    bfacenodes = np.array([[0, n - 1]], dtype=np.int32)
    bfaceregions = np.array([1, 2], dtype=np.int32)
    return Grid(coord, cellnodes, cellregions, bfacenodes, bfaceregions)


def _grid2d(X, Y):
    nx, ny = X.size, Y.size
    xx, yy = np.meshgrid(X, Y, indexing="xy")
    coord = np.stack([xx.ravel(), yy.ravel()])
    ix, iy = np.meshgrid(np.arange(nx - 1), np.arange(ny - 1), indexing="xy")
    p00 = (ix + nx * iy).ravel()
    p10, p01, p11 = p00 + 1, p00 + nx, p00 + nx + 1
    # two triangles per rectangle, interleaved: (p00,p10,p11), (p11,p01,p00)
    t1 = np.stack([p00, p10, p11])
    t2 = np.stack([p11, p01, p00])
    cellnodes = np.empty((3, 2 * p00.size), dtype=np.int32)
    cellnodes[:, 0::2] = t1
    cellnodes[:, 1::2] = t2
    cellregions = np.ones(cellnodes.shape[1], dtype=np.int32)
    bn, br = [], []
    i = np.arange(nx - 1)
    bn.append(np.stack([i, i + 1])); br.append(np.full(nx - 1, 1))                     # south
    j = np.arange(ny - 1)
    bn.append(np.stack([nx - 1 + nx * j, nx - 1 + nx * (j + 1)])); br.append(np.full(ny - 1, 2))  # east
    bn.append(np.stack([nx * (ny - 1) + i, nx * (ny - 1) + i + 1])); br.append(np.full(nx - 1, 3))  # north
    bn.append(np.stack([nx * j, nx * (j + 1)])); br.append(np.full(ny - 1, 4))           # west
    return Grid(coord, cellnodes, cellregions, np.concatenate(bn, axis=1),
                np.concatenate(br))


def _grid3d(X, Y, Z):
    nx, ny, nz = X.size, Y.size, Z.size
    zz, yy, xx = np.meshgrid(Z, Y, X, indexing="ij")
    coord = np.stack([xx.ravel(), yy.ravel(), zz.ravel()])

    def nid(i, j, k):
        return i + nx * (j + ny * k)

    ci, cj, ck = np.meshgrid(np.arange(nx - 1), np.arange(ny - 1), np.arange(nz - 1), indexing="ij")
    ci, cj, ck = (a.transpose(2, 1, 0).ravel() for a in (ci, cj, ck))  # x fastest
    base = np.stack([ci, cj, ck])
    steps = np.eye(3, dtype=np.int64)
    tets = []
    for perm in ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)):
        p = base.copy()
        verts = [nid(*p)]
        for a in perm:
            p = p + steps[a][:, None]
            verts.append(nid(*p))
        tets.append(np.stack(verts))
    cellnodes = np.stack(tets, axis=2).reshape(4, -1).astype(np.int32)  # 6 tets per brick, brick-major
    cellregions = np.ones(cellnodes.shape[1], dtype=np.int32)

    bn, br = [], []

    def face(fixed_axis, fixed_index, region):
        axes_ = [a for a in range(3) if a != fixed_axis]
        n_a = (nx, ny, nz)[axes_[0]]
        n_b = (nx, ny, nz)[axes_[1]]
        ia, ib = np.meshgrid(np.arange(n_a - 1), np.arange(n_b - 1), indexing="xy")
        ia, ib = ia.ravel(), ib.ravel()

        def pt(da, db):
            idx = [None, None, None]
            idx[fixed_axis] = np.full(ia.shape, fixed_index)
            idx[axes_[0]] = ia + da
            idx[axes_[1]] = ib + db
            return nid(*idx)

        lo, a1, b1, hi = pt(0, 0), pt(1, 0), pt(0, 1), pt(1, 1)
        tri = np.empty((3, 2 * ia.size), dtype=np.int64)
        tri[:, 0::2] = np.stack([lo, a1, hi])
        tri[:, 1::2] = np.stack([lo, b1, hi])
        bn.append(tri)
        br.append(np.full(tri.shape[1], region))

    face(1, 0, 1)          # south  y min
    face(0, nx - 1, 2)     # east   x max
    face(1, ny - 1, 3)     # north  y max
    face(0, 0, 4)          # west   x min
    face(2, 0, 5)          # bottom z min
    face(2, nz - 1, 6)     # top    z max
    return Grid(coord, cellnodes, cellregions, np.concatenate(bn, axis=1).astype(np.int32),
                np.concatenate(br).astype(np.int32))
