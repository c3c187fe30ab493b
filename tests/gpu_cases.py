"""Small problem definitions shared by the GPU parity tests: one per registered
physics, on grids small enough for the oracle to finish in well under a second."""
import os

import numpy as np


def lin(n):
    return np.array([i / n for i in range(n + 1)])


BIPOLAR = [1.0, 1.0, 1.0, 1.0, 1.0, 1.0e3, 0.5]  # lambda2, mu_n, mu_p, tau_n, tau_p, doping, V


def case(vfvm, name, seed=0):
    """Returns (grid, kind, params, nodedata, legacy(bf, bv) or None, state_fn, t, tstep, embed)."""
    rng = np.random.default_rng(seed)
    sg = vfvm.simplexgrid
    legacy = None
    nodedata = None
    tstep = np.inf
    t = 0.0
    embed = 0.0
    if name == "nlpoisson":
        g, kind, params = sg(lin(8), lin(8)), "nlpoisson", []
    elif name == "porous":
        g, kind, params, tstep = sg(lin(8), lin(8)), "porous", [], 1e-3
    elif name == "bipolar":
        g, kind, params, embed = sg(lin(4), lin(4), lin(4)), "bipolar", BIPOLAR, 0.3
    elif name == "rd2":
        g, kind, params = sg(lin(8), lin(8)), "rd2", [0.5, 2.0, 3.0]
    elif name == "kappa_exp":
        g, kind, params = sg(lin(8), lin(8)), "kappa_exp", [0.3]
        nodedata = np.exp(rng.normal(size=g.nnodes))
    elif name == "ex105":
        g, kind, params = sg(lin(10)), "ex105", [1e-3]
        legacy = (np.full((1, 2), 1e30), np.array([[0.0, 1.0]]))
    elif name == "ex106":
        g, kind, params, tstep = sg(np.array([(i - 10) / 10 for i in range(21)])), "ex106", [2.0], 1e-4
    elif name == "ex110":
        g, kind, params, tstep = sg(lin(20)), "ex110", [0.5, 0.5], 1e-2
        legacy = (np.full((2, 2), 1e30), np.array([[1.0, 0.0], [1.0, 0.0]]))
    elif name == "ex160":
        g, kind, params, tstep, t = sg(lin(20)), "ex160", [1e-3, -1.0, 5.0], 1e-3, 3e-3
    elif name == "ex207":
        g, kind, params, tstep = sg(lin(6), lin(6)), "ex207", [1e-2], 1e-2
        bf = np.zeros((1, 4)); bv = np.zeros((1, 4))
        bf[0, 1] = bf[0, 3] = 1e30; bv[0, 1] = bv[0, 3] = 0.1
        legacy = (bf, bv)
    elif name == "ex301":
        g, kind, params = sg(lin(3), lin(3), lin(3)), "ex301", []
        bf = np.zeros((1, 6)); bv = np.zeros((1, 6))
        bf[0, 4] = bf[0, 5] = 1e30
        legacy = (bf, bv)
    elif name == "ex440":
        g, kind, params = sg(lin(20)), "ex440", [3.0]
    elif name == "kappa_unstructured":  # Delaunay grid read from a SimplexGrid file
        g = sg(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "jittered_square.sg"))
        kind, params = "kappa_exp", [0.3]
        nodedata = np.exp(rng.normal(size=g.nnodes))
    elif name == "surface_heat2d":  # conducting surface layer on the right side (region 2)
        g, kind, params, tstep = sg(lin(8), lin(8)), "surface_heat", [1.0, 0.3, 0.5, 2.0, 10.0, 2], 1e-2
    elif name == "surface_heat3d":  # conducting surface layer on the bottom face (region 5)
        g, kind, params, tstep = sg(lin(4), lin(4), lin(4)), "surface_heat", [1.0, 0.3, 0.5, 2.0, 10.0, 5], 1e-2
    elif name == "edge_reaction2d":  # DevEx002: the unit source as an edge reaction -h^2/4
        g, kind, params = sg(lin(8), lin(8)), "edge_reaction", [1, 2]
    elif name == "edge_reaction3d":  # the edge reaction -(x_K - x_L)^2 / 2
        g, kind, params = sg(lin(3), lin(3), lin(3)), "edge_reaction", [2, 3]
    elif name == "joule_heat":  # Example206's callbacks on a 3 x 1 rectangle
        g, kind, params = sg(3 * lin(12), lin(4)), "joule_heat", [1.0, 1.0, 0.5, 1.0, 1.0]
    elif name == "ex161":  # Example161: three cell regions, bias ramp in time (mid-ramp here)
        import ex161_case
        g, kind, params = ex161_case.grid(vfvm), "ex161", ex161_case.PARAMS
        t, tstep = ex161_case.T_PRECOND + 0.5 * ex161_case.T_RAMP, 1e-6
    elif name == "ex430":  # Example430: Dirichlet value and coefficients from the parameter p
        g, kind, params = sg(lin(10), lin(10)), "ex430", [0.7]
    elif name == "outflow2d":  # pluto-examples/outflow.jl: outflow region 5 on part of the right side
        g = vfvm.bfacemask(sg(lin(10), lin(10)), [1, 0.3], [1, 0.7], 5)
        kind, params = "outflow", [1.0, 1.0, 0.5, 1.0, 4, 5]
    elif name.startswith("ex102_"):  # Example102's three fluxes; the upwind case with v < 0 (the other branch)
        mode = {"ex102_exp": 0, "ex102_upwind": 1, "ex102_central": 2}[name]
        g, kind, params = sg(lin(10)), "ex102", [0.01, -1.0 if mode == 1 else 1.0, mode]
        legacy = (np.full((1, 2), 1e30), np.array([[0.0, 1.0]]))
    elif name == "ex107":  # Example107: nonlinear storage (1e-10 + u)^(1/2)
        g, kind, params, tstep = sg(lin(20)), "ex107", [2.0, 1e-10], 1e-3
    elif name == "ex215":  # Example215: boundary reaction on region 2
        g, kind, params, tstep = sg(lin(8), lin(8)), "ex215", [1e-2, 1.0], 1e-2
    elif name == "laplace_dirichlet":
        g, kind, params = sg(lin(9)), "laplace_dirichlet", []
    else:
        raise KeyError(name)
    return dict(grid=g, kind=kind, params=params, nodedata=nodedata, legacy=legacy, t=t, tstep=tstep, embed=embed)


def random_state(c, nspec, rng):
    n = c["grid"].nnodes
    U = rng.uniform(0.2, 1.2, size=(nspec, n))
    if c["kind"] == "bipolar":
        U[0] = rng.uniform(-1.0, 1.0, size=n)
        U[1] = rng.uniform(0.5, 2.0, size=n)
        U[2] = rng.uniform(0.5, 2.0, size=n)
    if c["kind"] == "ex160":
        U[0] = rng.uniform(-1.0, 1.0, size=n)
        U[1] = rng.uniform(0.1, 0.9, size=n)
    return np.asfortranarray(U)


NAMES = ["nlpoisson", "porous", "bipolar", "rd2", "kappa_exp", "ex105", "ex106", "ex110", "ex160", "ex207",
         "ex301", "ex440", "laplace_dirichlet", "kappa_unstructured", "surface_heat2d", "surface_heat3d",
         "edge_reaction2d", "edge_reaction3d", "joule_heat", "ex161", "ex430", "outflow2d", "ex102_exp",
         "ex102_upwind", "ex102_central", "ex107", "ex215"]
