"""VoronoiFVM.jl solver oracle -- TEST INFRASTRUCTURE ONLY.

CPU FP64 restatement of the reference's Newton and time/embedding loops on top
of the C++ assembly restatement in ``vfvm_oracle.cpp``.  Only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` leg of ``bench.py`` use it,
as the checker; the package never imports it.

Restated reference code (paths relative to the reference project):

* ``solve_step!`` -- damped Newton, update-norm control, roundoff counter,
  monotonicity abort: ``src/vfvm_solver.jl:13-222``
* ``solve_transient!`` -- implicit Euler / parameter embedding with step
  control: ``src/vfvm_solver.jl:267-537``
* ``solve!`` dispatch: ``src/vfvm_solver.jl:551-617``
* ``SolverControl`` defaults: ``src/vfvm_solvercontrol.jl:13-270``
* ``fixed_timesteps!``: ``src/vfvm_solvercontrol.jl:320-327``

The reference's default sparse direct solver is UMFPACK through LinearSolve
(``src/vfvm_solver.jl:34-41``, ``src/vfvm_linsolve.jl:6-61``).  UMFPACK is not
available here; SuperLU (``scipy.sparse.linalg.splu``) stands in for it as the
sparse direct solve.
"""
from __future__ import annotations

import ctypes
import dataclasses
import math
import os
import subprocess
import time as _time

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

# coordinate systems (VFVM_COORD_* in include/vfvm_gb300.h)
COORD = {"cartesian": 0, "polar1d": 1, "spherical1d": 2, "cylindrical2d": 3}

# physics ids shared with include/vfvm_gb300.h
PHYS = {
    "ex105": 1, "ex106": 2, "ex110": 3, "ex160": 4, "ex207": 5, "ex301": 6, "ex440": 7,
    "laplace_dirichlet": 8, "nlpoisson": 11, "porous": 12, "bipolar": 13, "rd2": 14,
    "kappa_exp": 15, "surface_heat": 16, "boundary_species": 17, "edge_reaction": 18, "joule_heat": 19,
    "ex161": 20, "testfunction": 21, "ex430": 22, "outflow": 23, "ex210": 24,
    "ex102": 25, "ex107": 26, "ex115": 27, "ex215": 28, "ex220": 29, "ex203": 30,
}


def build(force: bool = False) -> str:
    """Compile the oracle shared library with the Makefile recipe next to this file."""
    src = os.path.join(_HERE, "vfvm_oracle.cpp")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.POINTER
        d, i32, i64 = ctypes.c_double, ctypes.c_int, ctypes.c_int64
        L.oracle_create.restype = ctypes.c_void_p
        L.oracle_create.argtypes = [i32, i32, P(d), i32, P(i32), P(i32), i32, P(i32), P(i32), i32,
                                    P(d), i32, P(d), i32, P(d), P(d), i32, i32]
        L.oracle_destroy.argtypes = [ctypes.c_void_p]
        L.oracle_set_cellwise.argtypes = [ctypes.c_void_p, i32]
        L.oracle_set_species.argtypes = [ctypes.c_void_p, i32, P(i32), i32, P(i32)]
        L.oracle_set_species.restype = i32
        L.oracle_nspec.argtypes = [ctypes.c_void_p]
        L.oracle_nedges.argtypes = [ctypes.c_void_p]
        L.oracle_ncandidates.argtypes = [ctypes.c_void_p]
        L.oracle_ncandidates.restype = i64
        L.oracle_factors.argtypes = [ctypes.c_void_p, P(d), P(d), P(i32)]
        L.oracle_bfacefactors.argtypes = [ctypes.c_void_p, P(d)]
        L.oracle_assemble.argtypes = [ctypes.c_void_p, P(d), P(d), d, d, d, P(d), i32]
        L.oracle_assemble.restype = i32
        L.oracle_csr.argtypes = [ctypes.c_void_p, P(i64), P(i32), P(d)]
        L.oracle_csr.restype = i64
        L.oracle_init_dirichlet.argtypes = [ctypes.c_void_p, P(d), d, d]
        L.oracle_integrate.argtypes = [ctypes.c_void_p, P(d), P(d), P(d), P(d)]
        L.oracle_mass_matrix.argtypes = [ctypes.c_void_p]
        L.oracle_parameter_derivatives.argtypes = [ctypes.c_void_p, P(d), d, d, d, P(d)]
        L.oracle_parameter_derivatives.restype = i32
        L.oracle_integrate_gradient.argtypes = [ctypes.c_void_p, P(d), P(d), i32, P(d), P(d)]
        L.oracle_integrate_gradient.restype = i32
        L.oracle_cellfactors.argtypes = [i32, P(d), P(i32), P(d), P(d)]
        L.oracle_bfacefactors_raw.argtypes = [i32, P(d), P(i32), P(d), P(d)]
        L.oracle_fbernoulli_pm.argtypes = [P(d), P(d), P(d), i64]
        _lib = L
    return _lib


def _p(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


class ConvergenceError(RuntimeError):
    """Newton did not converge (src/vfvm_logging_exceptions.jl)."""


class AssemblyError(RuntimeError):
    """NaN met during assembly (src/vfvm_assembly.jl:10-12)."""


@dataclasses.dataclass
class Control:
    """The SolverControl fields the oracle uses, with the reference defaults."""
    abstol: float = 1.0e-10
    reltol: float = 1.0e-10
    maxiters: int = 100
    tol_round: float = 1.0e-10
    tol_mono: float = 1.0e-3
    damp_initial: float = 1.0
    damp_growth: float = 1.2
    max_round: int = 1000
    updatecontrol: bool = True
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
    is_linear: bool = False


def fixed_timesteps(control: Control, dt: float, grow: float = 1.0) -> Control:
    """fixed_timesteps!, src/vfvm_solvercontrol.jl:320-327."""
    control.Δt = dt
    control.Δt_max = dt
    control.Δt_min = dt
    control.Δt_grow = grow
    control.Δu_opt = float(np.finfo(np.float64).max)
    return control


class OracleSystem:
    """Grid tables + physics id + parameters, evaluated by the C++ restatement."""

    def __init__(self, grid, physics, params=(), nodedata=None, bfactors=None, bvalues=None, assembly="edgewise",
                 region_species=None, bregion_species=None):
        """region_species (nspec x ncellregions) / bregion_species (nspec x
        nbregions): nonzero where enable_species! / enable_boundary_species!
        enabled a species (None for both: every species on every node)."""
        L = lib()
        self.physics_id = PHYS[physics] if isinstance(physics, str) else int(physics)
        self.grid = grid
        self.params = np.ascontiguousarray(params, dtype=np.float64)
        nd = 0
        self._nodedata = None
        if nodedata is not None:
            a = np.ascontiguousarray(np.atleast_2d(np.asarray(nodedata, dtype=np.float64)))
            if a.shape[1] != grid.nnodes:
                a = a.T.copy()
            nd = a.shape[0]
            self._nodedata = np.ascontiguousarray(a.T)  # nnodes x nd -> flat node-major
        nbreg = 0
        self._bf = self._bv = None
        if bfactors is not None:
            self._bf = np.asfortranarray(bfactors, dtype=np.float64)
            self._bv = np.asfortranarray(bvalues, dtype=np.float64)
            nbreg = self._bf.shape[1]
        g = grid
        # keep the marshalled tables alive for the duration of the call
        self._coord = np.ascontiguousarray(g.coord.T)
        self.h = L.oracle_create(
            g.dim, g.nnodes, _p(self._coord, ctypes.c_double),
            g.ncells, _p(np.ascontiguousarray(g.cellnodes.T), ctypes.c_int), _p(g.cellregions, ctypes.c_int),
            g.nbfaces, _p(np.ascontiguousarray(g.bfacenodes.T), ctypes.c_int), _p(g.bfaceregions, ctypes.c_int),
            self.physics_id, _p(self.params, ctypes.c_double), self.params.size,
            _p(self._nodedata, ctypes.c_double) if self._nodedata is not None else None, nd,
            _p(self._bf, ctypes.c_double) if self._bf is not None else None,
            _p(self._bv, ctypes.c_double) if self._bv is not None else None, nbreg,
            COORD[getattr(g, "coordsystem", "cartesian")])
        if not self.h:
            raise ValueError("oracle_create failed (unknown physics or bad dimension)")
        if assembly not in ("edgewise", "cellwise"):
            raise ValueError("assembly must be edgewise or cellwise")
        L.oracle_set_cellwise(self.h, int(assembly == "cellwise"))
        self.nspec = L.oracle_nspec(self.h)
        if region_species is not None or bregion_species is not None:
            rs = np.asfortranarray(np.zeros((self.nspec, 0)) if region_species is None else region_species,
                                   dtype=np.int32)
            bs = np.asfortranarray(np.zeros((self.nspec, 0)) if bregion_species is None else bregion_species,
                                   dtype=np.int32)
            self._species = (rs, bs)
            if L.oracle_set_species(self.h, rs.shape[1], _p(rs, ctypes.c_int), bs.shape[1], _p(bs, ctypes.c_int)):
                raise ValueError("a species is both a bulk and a boundary species, or no species is enabled")
        self.nnodes = g.nnodes
        self.n = self.nspec * self.nnodes
        self.tasm = 0.0
        self.tlin = 0.0

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.oracle_destroy(self.h)
            self.h = None

    # -- geometry
    def factors(self):
        L = lib()
        E = L.oracle_nedges(self.h)
        nv = np.zeros(self.nnodes)
        ef = np.zeros(E)
        en = np.zeros((E, 2), dtype=np.int32)
        L.oracle_factors(self.h, _p(nv, ctypes.c_double), _p(ef, ctypes.c_double), _p(en, ctypes.c_int))
        return nv, ef, en

    def nodevolumes(self):
        return self.factors()[0]

    def bfacefactors(self):
        """The node factors of every boundary face (dim x nbfaces, face after face)."""
        out = np.zeros(self.grid.dim * self.grid.nbfaces)
        lib().oracle_bfacefactors(self.h, _p(out, ctypes.c_double))
        return out

    # -- assembly
    def assemble(self, U, Uold=None, time=0.0, tstep=math.inf, embed=0.0, keep_pattern=False):
        """Return (F, J) with F flat in dof order K*nspec+i and J a scipy CSR matrix
        holding exactly the entries the reference would create."""
        L = lib()
        U = np.ascontiguousarray(U, dtype=np.float64).ravel()
        Uo = U if Uold is None else np.ascontiguousarray(Uold, dtype=np.float64).ravel()
        F = np.zeros(self.n)
        t0 = _time.perf_counter()
        rc = L.oracle_assemble(self.h, _p(U, ctypes.c_double), _p(Uo, ctypes.c_double), time, tstep, embed,
                               _p(F, ctypes.c_double), int(bool(keep_pattern)))
        if rc != 0:
            raise AssemblyError("trying to assemble NaN")
        nnz = L.oracle_csr(self.h, None, None, None)
        rp = np.zeros(self.n + 1, dtype=np.int64)
        ci = np.zeros(nnz, dtype=np.int32)
        vv = np.zeros(nnz)
        L.oracle_csr(self.h, _p(rp, ctypes.c_int64), _p(ci, ctypes.c_int), _p(vv, ctypes.c_double))
        self.tasm += _time.perf_counter() - t0
        J = sp.csr_matrix((vv, ci, rp), shape=(self.n, self.n))
        return F, J

    def parameter_derivatives(self, U, time=0.0, tstep=math.inf, embed=0.0):
        """dudp: the derivatives of the residual with respect to the physics'
        differentiable parameters at U, shape (npd, n)."""
        L = lib()
        U = np.ascontiguousarray(U, dtype=np.float64).ravel()
        npd = L.oracle_parameter_derivatives(self.h, _p(U, ctypes.c_double), time, tstep, embed, None)
        out = np.zeros((npd, self.n))
        if npd:
            L.oracle_parameter_derivatives(self.h, _p(U, ctypes.c_double), time, tstep, embed,
                                           _p(out, ctypes.c_double))
        return out

    def integrate_gradient(self, T, U, species=0):
        """Derivatives of the steady test-function current of `species` with
        respect to U (n values) and to the differentiable parameters."""
        L = lib()
        U = np.ascontiguousarray(U, dtype=np.float64).ravel()
        T = np.ascontiguousarray(T, dtype=np.float64).ravel()
        du = np.zeros(self.n)
        dp = np.zeros(4)
        npd = L.oracle_integrate_gradient(self.h, _p(T, ctypes.c_double), _p(U, ctypes.c_double), int(species),
                                          _p(du, ctypes.c_double), _p(dp, ctypes.c_double))
        return du, dp[:npd]

    def mass_matrix(self):
        """mass_matrix(state), src/vfvm_diffeq_interface.jl:60-112, as CSR."""
        L = lib()
        L.oracle_mass_matrix(self.h)
        nnz = L.oracle_csr(self.h, None, None, None)
        rp = np.zeros(self.n + 1, dtype=np.int64)
        ci = np.zeros(nnz, dtype=np.int32)
        vv = np.zeros(nnz)
        L.oracle_csr(self.h, _p(rp, ctypes.c_int64), _p(ci, ctypes.c_int), _p(vv, ctypes.c_double))
        return sp.csr_matrix((vv, ci, rp), shape=(self.n, self.n))

    def integrate(self, T, U, Uold=None, tstep=None):
        """Test-function integrals (src/vfvm_testfunctions.jl:125-380) of the
        flat solution U with test function T: a dict of per-species arrays
        flux, react, src, stor, oldstor, erea, and ``steady`` = flux + react -
        src + erea (integrate(system, T, U)) or, with Uold and tstep, that plus
        (stor - oldstor) / tstep (the implicit Euler step form)."""
        U = np.ascontiguousarray(U, dtype=np.float64).ravel()
        Uo = U if Uold is None else np.ascontiguousarray(Uold, dtype=np.float64).ravel()
        T = np.ascontiguousarray(T, dtype=np.float64).ravel()
        out = np.zeros(6 * self.nspec)
        lib().oracle_integrate(self.h, _p(T, ctypes.c_double), _p(U, ctypes.c_double), _p(Uo, ctypes.c_double),
                               _p(out, ctypes.c_double))
        parts = dict(zip(("flux", "react", "src", "stor", "oldstor", "erea"), out.reshape(6, self.nspec)))
        I = parts["flux"] + parts["react"] - parts["src"]
        if Uold is not None and tstep is not None:
            I = I + (parts["stor"] - parts["oldstor"]) / tstep
        parts["steady" if tstep is None else "step"] = I + parts["erea"]
        return parts

    def init_dirichlet(self, U, time=0.0, embed=0.0):
        lib().oracle_init_dirichlet(self.h, _p(U, ctypes.c_double), time, embed)
        return U

    # -- linear solve: sparse direct (UMFPACK substitute)
    def linsolve(self, J, F):
        t0 = _time.perf_counter()
        x = spla.splu(J.tocsc()).solve(F)
        self.tlin += _time.perf_counter() - t0
        return x


def testfunction(grid, bc0, bc1, assembly="edgewise"):
    """testfunction(TestFunctionFactory(system), bc0, bc1),
    src/vfvm_testfunctions.jl:38-108: the Laplace system of the factory with
    Dirichlet value -1 on the regions bc1 and 0 on bc0, its residual and matrix
    at 0, T = matrix \\ residual (T = 1 on bc1, 0 on bc0)."""
    nb = int(np.max(grid.bfaceregions))
    bf = np.zeros((1, nb))
    bv = np.zeros((1, nb))
    for r in bc1:
        bf[0, r - 1], bv[0, r - 1] = 1.0e30, -1.0
    for r in bc0:
        bf[0, r - 1], bv[0, r - 1] = 1.0e30, 0.0
    tsys = OracleSystem(grid, "testfunction", [], bfactors=bf, bvalues=bv, assembly=assembly)
    F, J = tsys.assemble(np.zeros(grid.nnodes), tstep=math.inf)
    return spla.splu(J.tocsc()).solve(F)


class NewtonHistory:
    def __init__(self):
        self.updatenorm = []
        self.l1normdiff = []
        self.niter = 0
        self.nlin = 0


def solve_step(osys: OracleSystem, oldsol, control: Control, time=0.0, tstep=math.inf, embed=0.0,
               linsolve=None):
    """solve_step!, src/vfvm_solver.jl:13-222.  Returns (solution, history)."""
    solution = np.array(oldsol, dtype=np.float64).ravel().copy()
    oldsol = np.asarray(oldsol, dtype=np.float64).ravel()
    osys.init_dirichlet(solution, time, embed)
    hist = NewtonHistory()
    linsolve = linsolve or osys.linsolve
    oldnorm = 1.0
    converged = False
    damp = 1.0
    rnorm = 0.0
    if not control.is_linear:
        damp = control.damp_initial
        rnorm = float(np.sum(np.abs(solution)))
    nround = 0
    tolx = 0.0
    niter = 1
    norm = 0.0
    while niter <= control.maxiters:
        F, J = osys.assemble(solution, oldsol, time, tstep, embed, keep_pattern=True)
        if not control.updatecontrol:
            # residual control (an extension; the reference controls the update
            # norm): max|F| over the rows without a Dirichlet penalty, and an
            # iterate that already meets the tolerance is returned unchanged
            free = np.abs(J.diagonal()) < 1.0e20  # rows without a Dirichlet penalty (1e30 on the diagonal)
            norm = float(np.max(np.abs(F[free]), initial=0.0))
            if not control.is_linear and (norm < control.abstol or norm < tolx):
                converged = True
                hist.niter = niter - 1
                break
        update = linsolve(J, F)
        hist.nlin += 1
        solution -= damp * update
        hist.niter = niter
        if control.is_linear:
            converged = True
            break
        damp = min(damp * control.damp_growth, 1.0)
        if control.updatecontrol:
            norm = float(np.max(np.abs(update)))
        if tolx == 0.0:
            tolx = norm * control.reltol
        dnorm = 1.0
        rnorm_new = float(np.sum(np.abs(solution)))
        if rnorm > 1.0e-50:
            dnorm = abs((rnorm - rnorm_new) / rnorm)
        nround = nround + 1 if dnorm < control.tol_round else 0
        hist.l1normdiff.append(dnorm)
        hist.updatenorm.append(norm)
        if niter > 1 and norm / oldnorm > 1.0 / control.tol_mono:
            converged = False
            break
        if norm < control.abstol or norm < tolx:
            converged = True
            break
        oldnorm = norm
        rnorm = rnorm_new
        if nround > control.max_round:
            converged = True
            break
        niter += 1
    if not converged:
        raise ConvergenceError("Newton did not converge")
    return solution, hist


def _isapprox(a, b, rtol=math.sqrt(np.finfo(float).eps), atol=0.0):
    return a == b or (math.isfinite(a) and math.isfinite(b) and abs(a - b) <= max(atol, rtol * max(abs(a), abs(b))))


def solve_transient(osys: OracleSystem, inival, lambdas, control: Control, transient=True, time=0.0,
                    delta=None, linsolve=None):
    """solve_transient!, src/vfvm_solver.jl:267-537.

    Returns (times, solutions, histories): the stored steps (store_all) including
    the initial value."""
    rd = lambda x: float(f"{x:.5g}")  # noqa: E731
    if transient:
        dl, dl_min, dl_max, dl_grow, dl_dec = control.Δt, control.Δt_min, control.Δt_max, control.Δt_grow, control.Δt_decrease
    else:
        dl, dl_min, dl_max, dl_grow, dl_dec = control.Δp, control.Δp_min, control.Δp_max, control.Δp_grow, control.Δp_decrease
    du_opt = control.Δu_opt
    du_max_factor = control.Δu_max_factor
    delta = delta or (lambda u, v, t, dt: float(np.max(np.abs(u - v))))
    solution = np.array(inival, dtype=np.float64).ravel().copy()
    oldsolution = solution.copy()
    hists = []
    if transient:
        ts = [float(lambdas[0])]
        sols = [solution.copy()]
        osys.init_dirichlet(solution, time, float(lambdas[0]))
    else:
        osys.init_dirichlet(solution, time, float(lambdas[0]))
        solution, h = solve_step(osys, solution, control, time, math.inf, float(lambdas[0]), linsolve)
        hists.append(h)
        oldsolution = solution.copy()
        ts = [float(lambdas[0])]
        sols = [solution.copy()]
    istep = 0
    solved = False
    lam = float(lambdas[0])
    lam0 = lam
    for i in range(len(lambdas) - 1):
        dl = max(dl, dl_min)
        lstart, lend = float(lambdas[i]), float(lambdas[i + 1])
        lam = lstart
        while lam < lend:
            solved = False
            lam0 = lam
            du = 0.0
            while not solved:
                solved = True
                errored = False
                try:
                    lam = lam0 + dl
                    if transient:
                        _t, _ts, _e = lam, dl, 0.0
                    else:
                        _t, _ts, _e = time, math.inf, lam
                    newsol, h = solve_step(osys, oldsolution, control, _t, _ts, _e, linsolve)
                except (ConvergenceError, AssemblyError, np.linalg.LinAlgError, RuntimeError) as err:
                    if not control.handle_exceptions:
                        raise RuntimeError(f"Solver problem at lambda={rd(lam)}, dlambda={rd(dl)}: {err}")
                    solved = False
                    errored = True
                else:
                    solution = newsol
                if solved:
                    du = float(delta(solution, oldsolution, lam, dl))
                    if du > du_max_factor * du_opt:
                        solved = False
                if not solved:
                    if _isapprox(dl, dl_min):
                        if not (control.force_first_step and istep == 0):
                            msg = f"At lambda={rd(lam)}: dlambda_min reached while du/du_opt={rd(du / du_opt)}"
                            if control.handle_exceptions:
                                break
                            raise RuntimeError(msg)
                        elif not errored:
                            solved = True
                        else:
                            if control.handle_exceptions:
                                break
                            raise RuntimeError("Convergence problem in first timestep")
                    else:
                        dl = max(dl_min, dl * dl_dec)
                        solution = oldsolution.copy()
            if solved:
                istep += 1
                hists.append(h)
                if control.store_all:
                    ts.append(lam)
                    sols.append(solution.copy())
                oldsolution = solution.copy()
                steps_to_go = math.ceil((lend - lam) / dl)
                lam_predict = lend - lam
                if steps_to_go < control.num_final_steps:
                    # Julia float division: 0/0 gives NaN (unused once lam reached lend)
                    lam_predict = (lend - lam) / steps_to_go if steps_to_go else math.nan
                if _isapprox(dl_max, dl_min):
                    lam_predict = dl_max
                if lam < lend:
                    dl = min(dl_max, dl * dl_grow, dl * du_opt / (du + 1.0e-14), lam_predict, lend - lam)
                    if _isapprox(lam + dl, lend, rtol=1.0e-15, atol=1.0e-15):
                        dl = lend - lam
            else:
                break
        if not control.store_all:
            ts.append(lam0)
            sols.append(solution.copy())
        if not solved:
            break
    return ts, sols, hists
