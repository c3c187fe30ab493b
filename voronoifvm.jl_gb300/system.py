"""Host-side mirror of the VoronoiFVM.jl interface for the assembly + Newton path.

Names, argument meaning and error behaviour follow the reference:

* ``System(grid, physics; species, ...)``  -- src/vfvm_system.jl:215-261
* ``Physics(...)``                         -- src/vfvm_physics.jl:67-182; here a
  registered device functor (``kind``) plus its data, because Julia closures
  cannot cross the C ABI
* ``boundary_dirichlet(sys, ispec, ireg, val)`` -- the system-level (legacy)
  Dirichlet data, src/vfvm_system.jl:329 and src/vfvm_assembly.jl:355-387
* ``enable_species(sys, ispec, regions)``, ``enable_boundary_species(sys, ispec,
  bregions)`` -- species restricted to cell or boundary regions,
  src/vfvm_system.jl:433-513
* ``SolverControl``, ``fixed_timesteps``   -- src/vfvm_solvercontrol.jl:13-327
* ``solve(sys; inival, control, times, embed, tstep, time, data)`` --
  src/vfvm_solver.jl:551-668
* ``evaluate_residual_and_jacobian``       -- src/vfvm_solver.jl:224-260
* ``unknowns``, ``nodevolumes``, ``integrate`` -- dense solution layout
  (src/vfvm_densesolution.jl:11-49) and src/vfvm_postprocess.jl:18-100,397-412
* ``eval_rhs``, ``eval_jacobian``, ``mass_matrix`` -- the ODE/DAE form,
  src/vfvm_diffeq_interface.jl:10-112
* ``parameter_derivatives`` -- the residual's derivatives with respect to the
  physics' differentiable parameters (the reference's dudp)
* ``TestFunctionFactory``, ``testfunction``, ``integrate(sys, T, U[, Uold,
  tstep])``, ``integrate_gradT_flux`` -- test-function currents,
  src/vfvm_testfunctions.jl:38-380
* exceptions ``ConvergenceError``, ``AssemblyError``, ``LinearSolverError``,
  ``EmbeddingError`` -- src/vfvm_logging_exceptions.jl:6-29

Solutions are ``numpy`` arrays of shape ``(nspec, nnodes)`` in Fortran order, so
their memory is the reference's dof order ``inode*nspec + ispec``.
"""
from __future__ import annotations

import ctypes
import dataclasses
import math
from typing import Optional, Sequence

import numpy as np
import scipy.sparse as sp

from . import _lib as L
from .grid import Grid

__all__ = ["Physics", "System", "SolverControl", "NewtonSolverHistory", "TransientSolution",
           "ConvergenceError", "AssemblyError", "LinearSolverError", "EmbeddingError",
           "boundary_dirichlet", "enable_species", "enable_boundary_species", "solve", "unknowns",
           "evaluate_residual_and_jacobian", "node_species",
           "fixed_timesteps", "nodevolumes", "integrate", "num_species", "TestFunctionFactory", "testfunction",
           "integrate_gradT_flux", "eval_rhs", "eval_jacobian", "mass_matrix", "parameter_derivatives"]

Dirichlet = 1.0e30  # src/vfvm_system.jl:329


class ConvergenceError(RuntimeError):
    """Newton's method did not converge."""


class AssemblyError(RuntimeError):
    """A NaN was assembled."""


class LinearSolverError(RuntimeError):
    """The linear solver failed."""


class EmbeddingError(RuntimeError):
    """Time/embedding step size fell to its minimum without convergence."""


def _raise(status: int, what: str = ""):
    if status == L.OK:
        return
    if status == L.ERR_CONVERGENCE:
        raise ConvergenceError(what or "Newton did not converge")
    if status == L.ERR_ASSEMBLY:
        raise AssemblyError(what or "trying to assemble NaN")
    if status == L.ERR_LINEAR:
        raise LinearSolverError(what or "linear solver error")
    if status == L.ERR_EMBEDDING:
        raise EmbeddingError(what or "minimal step size reached")
    if status == L.ERR_INPUT:
        raise ValueError(what or "invalid input to the CUDA library")
    raise RuntimeError(f"CUDA library error {status} {what}")


@dataclasses.dataclass
class Physics:
    """Selects a registered device physics functor and its data.

    ``kind``: one of ``_lib.PHYSICS_IDS``; ``data``: its parameter vector;
    ``nodedata``: optional per-node values (shape ``(nnodes,)`` or
    ``(nnodedata, nnodes)``); assign a new array to change them between solves
    (an array changed in place is not seen)."""
    kind: str
    data: Sequence[float] = ()
    nodedata: Optional[np.ndarray] = None

    @property
    def physics_id(self) -> int:
        try:
            return L.PHYSICS_IDS[self.kind]
        except KeyError:
            raise ValueError(f"unknown physics kind {self.kind!r}; known: {sorted(L.PHYSICS_IDS)}")


@dataclasses.dataclass
class SolverControl:
    """SolverControl with the reference defaults plus the device solver settings."""
    verbose: bool = False
    abstol: float = 1.0e-10
    reltol: float = 1.0e-10
    maxiters: int = 100
    tol_round: float = 1.0e-10
    tol_mono: float = 1.0e-3
    damp_initial: float = 1.0
    damp_growth: float = 1.2
    max_round: int = 1000
    updatecontrol: bool = True
    method_linear: str = "bicgstab"
    precon_linear: str = "ilu0"
    precision: str = "fp64"
    reltol_linear: float = 1.0e-4
    # The reference's 1e-8 floor belongs to its direct-solver default; with a
    # Krylov solve a floor ends Newton's update-norm control early, so the
    # device default is a purely relative (preconditioned) tolerance.
    abstol_linear: float = 0.0
    maxiters_linear: int = 100
    gmres_restart: int = 30
    Δp: float = 1.0
    Δp_max: float = 1.0
    Δp_min: float = 1.0e-3
    Δp_grow: float = 1.0
    Δp_decrease: float = 0.5
    Δt: float = 0.1
    Δt_max: float = 1.0
    Δt_min: float = 1.0e-3
    Δt_grow: float = 1.2
    Δt_decrease: float = 0.5
    Δu_opt: float = 0.1
    Δu_max_factor: float = 1.2
    force_first_step: bool = False
    num_final_steps: int = 5
    handle_exceptions: bool = False
    store_all: bool = True
    log: bool = False
    # device loop driver: "persistent" (one cooperative launch per solve), "graph"
    # (a CUDA graph of full-occupancy kernels) or "auto" (persistent for small systems)
    engine: str = "auto"
    # batched solves: CTAs per system (0: library default)
    team_ctas: int = 0
    # coarse-grid correction stage of the preconditioner: about this many coarse
    # unknowns (aggregates of nodes x species, at most 208); 0 = one-level only
    coarse: int = 0
    # batched solves on the sweep engine: end a Newton step's BiCGStab loop once at
    # most this many systems still iterate and they are at most a tenth of those
    # that entered the loop (they keep their current iterate; 0: off)
    batch_krylov_tail: int = 0
    # time / embedding step control of solve(times=...) / solve(embed=...):
    # "device" runs the whole step loop as one CUDA graph launch (the step
    # decisions made on the device, graph engine with BiCGStab); "host" decides
    # each step on the host around device Newton solves (any engine)
    step_control: str = "device"

    def to_c(self, is_linear: bool = False) -> L.Control_t:
        c = L.Control_t()
        c.abstol, c.reltol, c.maxiters = self.abstol, self.reltol, int(self.maxiters)
        c.tol_round, c.tol_mono = self.tol_round, self.tol_mono
        c.damp_initial, c.damp_growth, c.max_round = self.damp_initial, self.damp_growth, int(self.max_round)
        c.is_linear = int(bool(is_linear))
        c.updatecontrol = int(bool(self.updatecontrol))
        c.reltol_linear, c.abstol_linear, c.maxiters_linear = self.reltol_linear, self.abstol_linear, int(self.maxiters_linear)
        c.krylov = L.KRYLOV[self.method_linear]
        c.precon = L.PRECON[self.precon_linear]
        c.precision = L.PRECISION[self.precision]
        c.gmres_restart = int(self.gmres_restart)
        c.dt, c.dt_min, c.dt_max, c.dt_grow, c.dt_decrease = self.Δt, self.Δt_min, self.Δt_max, self.Δt_grow, self.Δt_decrease
        c.dp, c.dp_min, c.dp_max, c.dp_grow, c.dp_decrease = self.Δp, self.Δp_min, self.Δp_max, self.Δp_grow, self.Δp_decrease
        c.du_opt = min(self.Δu_opt, np.finfo(np.float64).max)
        c.du_max_factor = self.Δu_max_factor
        c.num_final_steps = int(self.num_final_steps)
        c.force_first_step = int(bool(self.force_first_step))
        c.handle_exceptions = int(bool(self.handle_exceptions))
        c.store_all = int(bool(self.store_all))
        c.engine = L.ENGINE[self.engine]
        c.team_ctas = int(self.team_ctas)
        c.coarse = int(self.coarse)
        c.batch_krylov_tail = int(self.batch_krylov_tail)
        return c


def fixed_timesteps(control: SolverControl, Δt: float, grow: float = 1.0) -> SolverControl:
    """fixed_timesteps!(control, Δt; grow), src/vfvm_solvercontrol.jl:320-327."""
    control.Δt = Δt
    control.Δt_max = Δt
    control.Δt_min = Δt
    control.Δt_grow = grow
    control.Δu_opt = np.finfo(np.float64).max
    return control


@dataclasses.dataclass
class NewtonSolverHistory:
    """Subset of NewtonSolverHistory (src/vfvm_history.jl:10-37) returned by the device solver."""
    nnewton: int = 0
    nlin: int = 0
    nsteps: int = 0
    updatenorm: float = 0.0
    resnorm: float = 0.0
    time: float = 0.0  # seconds
    status: int = 0    # 0, or the error code of the solve (batched solves report it per system)

    @classmethod
    def from_c(cls, h: L.History_t):
        return cls(h.nnewton, h.nlin, h.nsteps, h.updatenorm, h.resnorm, h.time_ms * 1e-3, h.status)


class TransientSolution:
    """Stored steps of a transient/embedding solve (src/vfvm_transientsolution.jl)."""

    def __init__(self, t, u, history=None):
        self.t = list(t)
        self.u = list(u)
        self.history = history

    def __len__(self):
        return len(self.t)

    def __getitem__(self, i):
        return self.u[i]


class System:
    """A finite-volume system on a grid with a registered device physics.

    The device context (tables, form factors, matrix pattern) is created on the
    first call that needs it and rebuilt when the legacy boundary data change.

    ``assembly``: the reference's :cellwise (its default) and :edgewise modes
    assemble the same operator -- the sum over cells of the cell-local terms --
    and differ only in summation order.  The device assembles both from
    edgewise tables (each edge's factors summed over its cells once, on the
    host), so every edge flux is evaluated once per edge instead of once per
    cell sharing it; the result agrees with the reference's cellwise summation
    to rounding.

    ``species``: the species enabled in every cell region (``None``: all of
    the physics' species).  ``enable_species`` / ``enable_boundary_species``
    restrict species to regions; the first such call on a system created with
    ``species=None`` starts from no species.

    ``unknown_storage``: the device keeps the dense layout (nspec unknowns per
    node) in both modes; a species a node does not carry is decoupled there by
    a unit row.  With ``:sparse`` the solutions read 0 on those dofs and
    ``evaluate_residual_and_jacobian`` returns the system of the carried dofs
    only -- what the reference's sparse storage holds."""

    def __init__(self, grid: Grid, physics: Physics, species: Optional[Sequence[int]] = None,
                 is_linear: bool = False, assembly: str = "edgewise", unknown_storage: str = "dense",
                 matrixtype: str = "sparse", valuetype=float, nparams: Optional[int] = None):
        if assembly not in ("edgewise", "cellwise"):
            raise ValueError("assembly must be :edgewise or :cellwise")
        if unknown_storage not in ("dense", "sparse"):
            raise ValueError("unknown_storage must be :dense or :sparse")
        # matrixtype (src/vfvm_system.jl:215-261): the reference's :banded and
        # :tridiagonal choices for 1D select its direct solver; the device keeps
        # one block-sparse matrix and its Krylov solve for every choice
        if matrixtype not in ("sparse", "banded", "tridiagonal", "default", "auto"):
            raise ValueError("matrixtype must be :sparse, :banded, :tridiagonal or :default")
        if valuetype not in (float, np.float64):
            raise ValueError("the device computes in Float64 (valuetype = Float64)")
        npd = L.physics_npd(physics.physics_id)
        if nparams is not None and int(nparams) != npd:
            raise ValueError(f"physics {physics.kind!r} has {npd} differentiable parameter(s), not {nparams}")
        self.matrixtype = matrixtype
        self.nparams = npd
        self.grid = grid
        self.physics = physics
        self.nspec = L.PHYSICS_NSPEC[physics.physics_id]
        self.is_linear = is_linear
        self.assembly = assembly
        self.unknown_storage = unknown_storage
        nb = max(grid.num_bfaceregions, 1)
        self.boundary_factors = np.zeros((self.nspec, nb), order="F")
        self.boundary_values = np.zeros((self.nspec, nb), order="F")
        # region_species (nspec x cell regions) / bregion_species (nspec x
        # boundary regions): None = every species on every node
        self.region_species = None
        self.bregion_species = None
        self.species = list(range(1, self.nspec + 1)) if species is None else list(species)
        if species is not None:
            enable_species(self, self.species, None)
        self._ctx = None
        self._ctx_key = None
        self._nodedata_id = None
        self._keep = None

    # -- context management
    def _marshal(self):
        g = self.grid
        keep = {}
        keep["coord"] = np.asfortranarray(g.coord)  # dim x nnodes column-major
        keep["cellnodes"] = np.asfortranarray(g.cellnodes, dtype=np.int32)
        keep["cellregions"] = np.ascontiguousarray(g.cellregions, dtype=np.int32)
        keep["bfacenodes"] = np.asfortranarray(g.bfacenodes, dtype=np.int32)
        keep["bfaceregions"] = np.ascontiguousarray(g.bfaceregions, dtype=np.int32)
        gt = L.Grid_t(g.dim, g.nnodes, g.ncells, g.nbfaces,
                      L.ptr(keep["coord"]), L.ptr(keep["cellnodes"], L.c_i32), L.ptr(keep["cellregions"], L.c_i32),
                      L.ptr(keep["bfacenodes"], L.c_i32), L.ptr(keep["bfaceregions"], L.c_i32),
                      L.COORD[g.coordsystem])
        params = np.ascontiguousarray(self.physics.data, dtype=np.float64)
        if params.size == 0:
            params = np.zeros(1)
        keep["params"] = params
        nd = 0
        ndp = None
        if self.physics.nodedata is not None:
            a = np.asarray(self.physics.nodedata, dtype=np.float64)
            a = a.reshape(-1, g.nnodes) if a.ndim == 1 else a
            if a.shape[1] != g.nnodes:
                raise ValueError("nodedata must have nnodes columns")
            keep["nodedata"] = np.ascontiguousarray(a.T)  # node-major
            nd = a.shape[0]
            ndp = L.ptr(keep["nodedata"])
        keep["bf"] = np.asfortranarray(self.boundary_factors)
        keep["bv"] = np.asfortranarray(self.boundary_values)
        pt = L.Physics_t(self.physics.physics_id, len(self.physics.data), L.ptr(params), nd, ndp,
                         keep["bf"].shape[1], L.ptr(keep["bf"]), L.ptr(keep["bv"]))
        if self.region_species is not None:
            keep["rs"] = np.asfortranarray(self.region_species, dtype=np.int32)
            keep["bs"] = np.asfortranarray(self.bregion_species, dtype=np.int32)
            pt.ncellregions_species = keep["rs"].shape[1]
            pt.region_species = L.ptr(keep["rs"], L.c_i32)
            pt.nbregions_species = keep["bs"].shape[1]
            pt.bregion_species = L.ptr(keep["bs"], L.c_i32)
        return gt, pt, keep

    @property
    def ctx(self):
        nd = self.physics.nodedata
        key = (self.grid.coordsystem, self.boundary_factors.tobytes(), self.boundary_values.tobytes(),
               None if nd is None else np.shape(nd),
               None if self.region_species is None else (self.region_species.tobytes(),
                                                         self.bregion_species.tobytes()))
        if self._ctx is None or key != self._ctx_key:
            lib = L.load()
            self.close()
            gt, pt, keep = self._marshal()
            status = ctypes.c_int(0)
            h = lib.vfvm_create(ctypes.byref(gt), ctypes.byref(pt), ctypes.byref(status))
            if not h:
                _raise(status.value or L.ERR_INPUT, "vfvm_create failed")
            self._ctx, self._ctx_key, self._keep = h, key, keep
            self._params = tuple(self.physics.data)
            self._nodedata_id = id(nd)
        else:
            if tuple(self.physics.data) != self._params:
                self._set_params(self.physics.data)
            if nd is not None and id(nd) != self._nodedata_id:
                # same shape, new values: upload them into the existing context
                a = np.asarray(nd, dtype=np.float64)
                a = a.reshape(-1, self.grid.nnodes) if a.ndim == 1 else a
                h = np.ascontiguousarray(a.T)
                _raise(L.load().vfvm_set_nodedata(self._ctx, L.ptr(h), a.shape[0]), "vfvm_set_nodedata")
                self._nodedata_id = id(nd)
        return self._ctx

    def _set_params(self, data):
        p = np.ascontiguousarray(data, dtype=np.float64)
        _raise(L.load().vfvm_set_params(self._ctx, L.ptr(p), p.size), "vfvm_set_params")
        self._params = tuple(data)

    def close(self):
        if self._ctx is not None:
            L.load().vfvm_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- sizes
    @property
    def nnodes(self) -> int:
        return self.grid.nnodes

    @property
    def ndofs(self) -> int:
        return self.nspec * self.grid.nnodes

    def info(self) -> dict:
        out = np.zeros(8, dtype=np.int64)
        _raise(L.load().vfvm_info(self.ctx, L.ptr(out, L.c_i64)))
        return dict(nspec=int(out[0]), nnodes=int(out[1]), nedges=int(out[2]), nnz=int(out[3]),
                    nblocks=int(out[4]), ncolors=int(out[5]), dim=int(out[6]), multiregion=bool(out[7]))

    def pattern(self):
        inf = self.info()
        rp = np.zeros(self.ndofs + 1, dtype=np.int64)
        ci = np.zeros(inf["nnz"], dtype=np.int32)
        _raise(L.load().vfvm_pattern(self.ctx, L.ptr(rp, L.c_i64), L.ptr(ci, L.c_i32)))
        return rp, ci


def num_species(sys: System) -> int:
    return sys.nspec


def boundary_dirichlet(sys: System, ispec: int, ireg: int, val: float):
    """boundary_dirichlet!(sys, ispec, ireg, val): system-level Dirichlet data
    (species and region numbers 1-based as in the reference)."""
    nb = max(sys.boundary_factors.shape[1], ireg)
    if nb > sys.boundary_factors.shape[1]:
        bf = np.zeros((sys.nspec, nb), order="F")
        bv = np.zeros((sys.nspec, nb), order="F")
        bf[:, :sys.boundary_factors.shape[1]] = sys.boundary_factors
        bv[:, :sys.boundary_values.shape[1]] = sys.boundary_values
        sys.boundary_factors, sys.boundary_values = bf, bv
    sys.boundary_factors[ispec - 1, ireg - 1] = Dirichlet
    sys.boundary_values[ispec - 1, ireg - 1] = val


def _species_tables(sys: System):
    if sys.region_species is None:
        g = sys.grid
        nreg = int(np.max(g.cellregions)) if g.ncells else 1
        nb = max(int(np.max(g.bfaceregions)) if g.nbfaces else 1, 1)
        sys.region_species = np.zeros((sys.nspec, nreg), dtype=np.int32, order="F")
        sys.bregion_species = np.zeros((sys.nspec, nb), dtype=np.int32, order="F")
    return sys.region_species, sys.bregion_species


def enable_species(sys: System, ispec, regions=None):
    """enable_species!(system, ispec, regions) (src/vfvm_system.jl:433-480): add
    species ``ispec`` (1-based; an int or a list) to the cell regions
    ``regions`` (1-based; None: all).  A species cannot be both a bulk and a
    boundary species (the reference's DomainError, raised as ValueError)."""
    rs, bs = _species_tables(sys)
    regs = range(1, rs.shape[1] + 1) if regions is None else list(regions)
    for i in ([ispec] if np.isscalar(ispec) else list(ispec)):
        i = int(i)
        if not 1 <= i <= sys.nspec:
            raise ValueError(f"species {i} outside 1..{sys.nspec} of this physics")
        if bs[i - 1].any():
            raise ValueError(f"species {i} is already a boundary species")
        for r in regs:
            if not 1 <= int(r) <= rs.shape[1]:
                raise ValueError(f"cell region {r} outside 1..{rs.shape[1]}")
            rs[i - 1, int(r) - 1] = 1
    return sys


def enable_boundary_species(sys: System, ispec: int, bregions):
    """enable_boundary_species!(system, ispec, bregions) (src/vfvm_system.jl:483-513):
    add species ``ispec`` to the boundary regions ``bregions`` (1-based)."""
    rs, bs = _species_tables(sys)
    i = int(ispec)
    if not 1 <= i <= sys.nspec:
        raise ValueError(f"species {i} outside 1..{sys.nspec} of this physics")
    if rs[i - 1].any():
        raise ValueError(f"species {i} is already a bulk species")
    for r in bregions:
        if not 1 <= int(r) <= bs.shape[1]:
            raise ValueError(f"boundary region {r} outside 1..{bs.shape[1]}")
        bs[i - 1, int(r) - 1] = 1
    return sys


def node_species(sys: System) -> np.ndarray:
    """Boolean (nspec, nnodes): whether node K carries species i -- the
    reference's node_dof (isnodespecies, src/vfvm_system.jl:765)."""
    g = sys.grid
    out = np.zeros((sys.nspec, g.nnodes), dtype=bool)
    if sys.region_species is None:
        out[...] = True
        return out
    rs, bs = sys.region_species != 0, sys.bregion_species != 0
    for r in range(rs.shape[1]):
        nodes = np.unique(g.cellnodes[:, g.cellregions == r + 1])
        out[np.ix_(rs[:, r], nodes)] = True
    for r in range(bs.shape[1]):
        nodes = np.unique(g.bfacenodes[:, g.bfaceregions == r + 1])
        out[np.ix_(bs[:, r], nodes)] = True
    return out


def _sparse_view(sys: System, U: np.ndarray) -> np.ndarray:
    """A solution as the reference's sparse storage reads it: 0 on the dofs
    a node does not carry."""
    if sys.unknown_storage == "sparse" and sys.region_species is not None:
        U = np.array(U, order="F")
        U[~node_species(sys)] = 0.0
    return U


def unknowns(sys: System, inival=0.0) -> np.ndarray:
    """Dense solution array (nspec, nnodes), Fortran order."""
    U = np.empty((sys.nspec, sys.nnodes), order="F")
    U[...] = inival
    return U


def _flat(U, sys: System) -> np.ndarray:
    a = np.asarray(U, dtype=np.float64)
    if a.ndim == 0:
        return np.full(sys.ndofs, float(a))
    if a.shape == (sys.nspec, sys.nnodes):
        return np.ascontiguousarray(a.ravel(order="F"))
    if a.size == sys.ndofs:
        return np.ascontiguousarray(a.ravel())
    raise ValueError(f"expected {sys.ndofs} unknowns, got shape {a.shape}")


def _shape(x: np.ndarray, sys: System) -> np.ndarray:
    return x.reshape((sys.nspec, sys.nnodes), order="F")


def evaluate_residual_and_jacobian(sys: System, u, t: float = 0.0, tstep: float = math.inf, embed: float = 0.0,
                                   init_dirichlet: bool = False, uold=None):
    """Residual (nspec, nnodes) and Jacobian (scipy CSR) at u, computed on the GPU."""
    lib = L.load()
    h = sys.ctx
    U = _flat(u, sys).copy()
    if init_dirichlet:
        _raise(lib.vfvm_init_dirichlet(h, L.ptr(U), t, embed))
    Uo = U if uold is None else _flat(uold, sys)
    rp, ci = sys.pattern()
    F = np.zeros(sys.ndofs)
    vals = np.zeros(ci.size)
    _raise(lib.vfvm_assemble(h, L.ptr(U), L.ptr(Uo), t, tstep, embed, L.ptr(F), L.ptr(vals)))
    J = sp.csr_matrix((vals, ci, rp), shape=(sys.ndofs, sys.ndofs))
    if sys.unknown_storage == "sparse" and sys.region_species is not None:
        # the carried dofs only (node-major, species ascending: the sparse dof order)
        act = np.flatnonzero(node_species(sys).ravel(order="F"))
        return F[act], J[act][:, act].tocsr()
    return _shape(F, sys), J


def eval_rhs(sys: System, u, t: float = 0.0) -> np.ndarray:
    """eval_rhs!(du, u, state, t) (src/vfvm_diffeq_interface.jl:29-34): the ODE
    right hand side -F(u) with the residual at tstep = Inf (the time
    derivative is the ODE solver's), shape (nspec, nnodes)."""
    F, _ = evaluate_residual_and_jacobian(sys, u, t=t, tstep=math.inf)
    return -F


def eval_jacobian(sys: System, u, t: float = 0.0):
    """eval_jacobian!(J, u, state, t) (src/vfvm_diffeq_interface.jl:42-48): -J."""
    _, J = evaluate_residual_and_jacobian(sys, u, t=t, tstep=math.inf)
    return -J


def parameter_derivatives(sys: System, u, t: float = 0.0, tstep: float = math.inf, embed: float = 0.0) -> np.ndarray:
    """dudp (src/vfvm_assembly.jl:116-120,194-198,403-405,...): dF/dp_k at u for
    the physics' differentiable parameters (the first npd entries of its
    parameter block), computed on the device; shape (npd, nspec, nnodes).
    With F(u(p), p) = 0, du/dp = -J^-1 dudp."""
    lib = L.load()
    U = _flat(u, sys)
    npd = ctypes.c_int32(0)
    _raise(lib.vfvm_parameter_derivatives(sys.ctx, L.ptr(U), t, tstep, embed, None, ctypes.byref(npd)),
           "vfvm_parameter_derivatives")
    out = np.zeros((npd.value, sys.ndofs))
    if npd.value:
        _raise(lib.vfvm_parameter_derivatives(sys.ctx, L.ptr(U), t, tstep, embed, L.ptr(out), ctypes.byref(npd)),
               "vfvm_parameter_derivatives")
    return np.stack([_shape(r, sys) for r in out]) if npd.value else out.reshape(0, sys.nspec, sys.nnodes)


def mass_matrix(sys: System):
    """mass_matrix(state) (src/vfvm_diffeq_interface.jl:60-112): the storage
    Jacobian at U = 0 on the device, as a scipy CSR matrix in the scalar
    pattern (a diagonal one for storage u)."""
    rp, ci = sys.pattern()
    vals = np.zeros(ci.size)
    _raise(L.load().vfvm_mass_matrix(sys.ctx, L.ptr(vals)), "vfvm_mass_matrix")
    return sp.csr_matrix((vals, ci, rp), shape=(sys.ndofs, sys.ndofs))


def nodevolumes(sys: System) -> np.ndarray:
    """Voronoi node volumes (src/vfvm_postprocess.jl:397-412)."""
    nv = np.zeros(sys.nnodes)
    _raise(L.load().vfvm_geometry(sys.ctx, L.ptr(nv), None, None))
    return nv


def edgefactors(sys: System):
    inf = sys.info()
    ef = np.zeros(inf["nedges"])
    en = np.zeros((inf["nedges"], 2), dtype=np.int32)
    _raise(L.load().vfvm_geometry(sys.ctx, None, L.ptr(ef), L.ptr(en, L.c_i32)))
    return ef, en


def _tf_parts(sys: System, T, U, Uold=None):
    """The six per-species test-function sums of vfvm_integrate, evaluated on
    the device at time 0 and embedding 1 (as the reference's Node(system, 0, 1))."""
    Tv = np.ascontiguousarray(np.asarray(T, dtype=np.float64).ravel())
    if Tv.size != sys.nnodes:
        raise ValueError("the test function needs one value per node")
    Uf = _flat(U, sys)
    Uo = None if Uold is None else _flat(Uold, sys)
    out = np.zeros(6 * sys.nspec)
    _raise(L.load().vfvm_integrate(sys.ctx, L.ptr(Tv), L.ptr(Uf), None if Uo is None else L.ptr(Uo), 0.0, 1.0,
                                   L.ptr(out)), "vfvm_integrate")
    return dict(zip(("flux", "react", "src", "stor", "oldstor", "erea"), out.reshape(6, sys.nspec)))


def integrate(sys: System, U, Ustate=None, Uold=None, tstep=None) -> np.ndarray:
    """integrate(system, U): per species sum of node volume x value
    (single cell region), src/vfvm_postprocess.jl:94-100.

    integrate(system, T, U) with a test function T (``testfunction``): the
    steady current flux + reaction - source (+ edge reaction), and
    integrate(system, T, U, Uold, tstep) the implicit Euler step form, which adds
    (storage(U) - storage(Uold)) / tstep (src/vfvm_testfunctions.jl:125-205)."""
    if Ustate is None:
        nv = nodevolumes(sys)
        return _shape(_flat(U, sys), sys) @ nv
    parts = _tf_parts(sys, U, Ustate, Uold)
    current = parts["flux"] + parts["react"] - parts["src"] + parts["erea"]
    if Uold is not None and tstep is not None:
        current = current + (parts["stor"] - parts["oldstor"]) / tstep
    return current


def integrate_gradT_flux(sys: System, T, U) -> np.ndarray:
    """integrate_∇TxFlux(system, T, U) (src/vfvm_testfunctions.jl:283-330): per
    species sum over the edges of fac * flux(U) * (T_first - T_second)."""
    return _tf_parts(sys, T, U)["flux"]


class TestFunctionFactory:
    """TestFunctionFactory(system) (src/vfvm_testfunctions.jl:38-50): the
    Laplace system (flux u_K - u_L, storage u) on the system's grid."""

    def __init__(self, system: System, control: Optional[SolverControl] = None):
        self.system = system
        self.tfsystem = System(system.grid, Physics("testfunction"), is_linear=True)
        self.control = control if control is not None else SolverControl(reltol_linear=1e-13,
                                                                           maxiters_linear=2000)


def testfunction(factory: TestFunctionFactory, bc0, bc1) -> np.ndarray:
    """testfunction(factory, B_0, B_1) (src/vfvm_testfunctions.jl:53-108):
    -Laplace T = 0 with T = 0 on the boundary regions bc0, T = 1 on bc1 and
    no flux elsewhere, solved on the device.  Returns T (one value per node)."""
    tf = factory.tfsystem
    tf.boundary_factors[...] = 0.0
    tf.boundary_values[...] = 0.0
    for r in bc1:
        boundary_dirichlet(tf, 1, int(r), 1.0)
    for r in bc0:
        boundary_dirichlet(tf, 1, int(r), 0.0)
    return np.asarray(solve(tf, inival=0.0, control=factory.control)).ravel().copy()


def solve(sys: System, inival=0.0, control: Optional[SolverControl] = None, times=None, embed=None,
          tstep: float = math.inf, time: float = 0.0, data=None, **kwargs):
    """solve(system; kwargs...) (src/vfvm_solver.jl:551-668).

    Stationary (or one implicit Euler step with ``tstep``) -> solution array with
    ``.history``-like attribute via the returned ``(U)``; with ``times`` or
    ``embed`` -> TransientSolution."""
    control = control if control is not None else SolverControl()
    for k, v in kwargs.items():
        if not hasattr(control, k):
            raise TypeError(f"unknown solve keyword {k!r}")
        setattr(control, k, v)
    if data is not None:
        sys.physics.data = tuple(data)
    lib = L.load()
    h = sys.ctx
    U0 = _flat(inival, sys)
    c = control.to_c(sys.is_linear)
    hist = L.History_t()
    if times is not None or embed is not None:
        lambdas = np.ascontiguousarray(times if times is not None else embed, dtype=np.float64)
        transient = times is not None
        t0 = float(lambdas[0]) if transient else time
        max_store = 100000 if control.store_all else max(len(lambdas), 1)
        max_store = min(max_store, max(16, int(2.0e9 // (8 * sys.ndofs))))
        store = np.zeros((max_store, sys.ndofs))
        tst = np.zeros(max_store)
        nst = ctypes.c_int32(0)
        on_device = (control.step_control == "device" and control.method_linear == "bicgstab"
                     and bool(np.all(np.diff(lambdas) > 0)))
        if on_device:
            syncs = ctypes.c_int32(0)
            rc = lib.vfvm_evolve_device(h, ctypes.byref(c), L.ptr(U0), L.ptr(lambdas), lambdas.size, int(transient),
                                        t0, L.ptr(store), L.ptr(tst), max_store, ctypes.byref(nst), ctypes.byref(hist),
                                        ctypes.byref(syncs))
            solve.last_host_syncs = int(syncs.value)
            _raise(rc, "vfvm_evolve_device")
        else:
            rc = lib.vfvm_evolve(h, ctypes.byref(c), L.ptr(U0), L.ptr(lambdas), lambdas.size, int(transient), t0,
                                 L.ptr(store), L.ptr(tst), max_store, ctypes.byref(nst), ctypes.byref(hist))
            solve.last_host_syncs = None
            _raise(rc, "vfvm_evolve")
        n = nst.value
        return TransientSolution(tst[:n].tolist(),
                                 [_sparse_view(sys, _shape(store[i].copy(), sys)) for i in range(n)],
                                 NewtonSolverHistory.from_c(hist))
    U = np.zeros(sys.ndofs)
    rc = lib.vfvm_solve(h, ctypes.byref(c), L.ptr(U0), L.ptr(U), time, tstep, 0.0, ctypes.byref(hist))
    _raise(rc, "vfvm_solve")
    out = _sparse_view(sys, _shape(U, sys))
    solve.last_history = NewtonSolverHistory.from_c(hist)
    return out


solve.last_history = None
solve.last_host_syncs = None  # host synchronisations of the last device-controlled evolution
