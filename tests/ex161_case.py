"""examples/Example161_BipolarDriftDiffusionCurrent.jl as a test case, shared by
the oracle golden test and the GPU test.

The grid (:35-51): three glued uniform pieces of n, 4n and 2n points on
[0, 0.5], [0.5, 4.5], [4.5, 5] (ExtendableGrids' glue drops the repeated
junction point), cell regions 1/2/3 by cellmask! on those intervals, boundary
regions 1 (x = 0) and 2 (x = 5).  Physics constants :59-76, solver control
:164-173, three solve phases :175-188, the test function between boundary
regions 1 and 2 and the current sum(I2) :196-220.
"""
import math

import numpy as np

N = 20
H1, H2, H3 = 0.5, 4.0, 0.5
T_PRECOND, T_RAMP, T_EXT = 5.0, 1.0e-5, 75.0
# Cn, Cp, Ca, En, Ep, mu_n, mu_p, lambda, tPrecond, tRamp, tExt, Vprecond, VExt, DirichletVal
PARAMS = [10.0, 10.0, 0.0, 1.0, 0.0, 10.0, 10.0, 1.0e-1, T_PRECOND, T_RAMP, T_EXT, 1.0, -3.0, 0.0]


def glue(a, b, tol=1e-10):
    return np.concatenate([a, b[1:]]) if abs(a[-1] - b[0]) < tol else np.concatenate([a, b])


def coords(n=N):
    ht = H1 + H2 + H3
    c1 = np.linspace(0.0, H1, n)
    c2 = np.linspace(H1, H1 + H2, 4 * n)
    c3 = np.linspace(H1 + H2, ht, 2 * n)
    return glue(glue(c1, c2), c3)


def grid(vfvm, n=N):
    X = coords(n)
    g = vfvm.simplexgrid(X)
    xc = g.coord[0, g.cellnodes].mean(axis=0)
    cr = np.where(xc < H1, 1, np.where(xc < H1 + H2, 2, 3)).astype(np.int32)
    return vfvm.Grid(g.coord, g.cellnodes, cr, g.bfacenodes, g.bfaceregions)


def inival(X):
    """inival2 (:175-179): phi_n = phi_p = 0, psi linear between asinh(Cn/2) and asinh(-Cp/2)."""
    ht = H1 + H2 + H3
    u = np.zeros((3, X.size))
    u[2] = math.asinh(10.0 / 2) + ((math.asinh(-10.0 / 2) + 0.0) - math.asinh(10.0 / 2)) / ht * X
    return u


def control_fields():
    """The SolverControl changes of :164-173, then of each phase."""
    base = dict(max_round=3, damp_initial=0.9, damp_growth=1.61, abstol=1e-5, reltol=1e-5, tol_round=1e-5)
    phases = [((0.0, T_PRECOND), {}),
              ((T_PRECOND, T_PRECOND + T_RAMP), {"Δt_min": 1e-8, "Δt": 1e-8}),
              ((T_PRECOND + T_RAMP, T_PRECOND + T_RAMP + T_EXT), {"Δt_min": 1e-10, "Δt": 1e-10, "Δt_grow": 1.7})]
    return base, phases


def current_sum(osys, tf, times, sols):
    """sum(I2) over the steps of the last phase (:200-220): the electron and hole
    flux integrals plus the displacement current of psi."""
    total = 0.0
    for k in range(1, len(times)):
        dt = times[k] - times[k - 1]
        e_new = osys.integrate(tf, sols[k])["flux"]
        e_old = osys.integrate(tf, sols[k - 1])["flux"]
        total += e_new[0] + e_new[1] + (e_new[2] - e_old[2]) / dt
    return total
