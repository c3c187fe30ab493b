"""GPU parity at the benchmark configurations' own sizes.

The other parity tests run on small grids; these run the assembly and the
Newton solve on the grids the benchmark configurations name, against the
oracle on the same inputs:

* configuration 1, nonlinear Poisson on 65 x 65 points: assembly parity and
  one full Newton solve (<= 1e-8 relative to the oracle's FP64 solution);
* configuration 2, porous medium on 513 x 513 points: one transient assembly
  at a random state, in the FP64 form (residual and Jacobian) and in the mixed
  form (its FP64 residual), and two implicit Euler steps of the mixed form;
* configuration 3, bipolar drift-diffusion on the tetrahedral grid of 64^3
  points (262144 nodes, 3 species): one assembly at a random state at
  embedding parameter 0.5;
* configuration 4, two-species reaction-diffusion: a batch of uneven grids
  whose largest member has the configuration's largest side, 257, solved by
  the batched solver; every member agrees with its own oracle solve.

Tolerances as in the small-grid tests: pattern bit-exact, residual and
Jacobian 1e-12 row-relative, solutions 1e-8 relative.
"""
import ctypes

import numpy as np
import pytest

from gpu_cases import BIPOLAR

pytestmark = pytest.mark.gpu
TOL = 1e-12
SOL_TOL = 1e-8


def grid(vfvm, n, dim):
    X = np.linspace(0.0, 1.0, n)
    return vfvm.simplexgrid(*([X] * dim))


def check_assembly(J, F, Jo, Fo, U):
    """Pattern bit-exact; F and J within TOL of the magnitude of the terms summed
    into each row (the same measure as the small-grid assembly tests)."""
    Jo.sort_indices()
    assert np.array_equal(J.indptr, Jo.indptr), "row pointers differ"
    assert np.array_equal(J.indices, Jo.indices), "column indices differ"
    absJ = abs(Jo)
    rowscale = np.maximum(np.abs(Fo), absJ @ np.abs(U))
    err = np.abs(F - Fo)
    assert np.all(err <= TOL * rowscale + 1e-300), f"max rel residual err {np.max(err / np.maximum(rowscale, 1e-300)):.3e}"
    rowmax = np.maximum.reduceat(np.abs(Jo.data), Jo.indptr[:-1])
    rows = np.repeat(np.arange(Jo.shape[0]), np.diff(Jo.indptr))
    jerr = np.abs(J.data - Jo.data)
    assert np.all(jerr <= TOL * rowmax[rows] + 1e-300), \
        f"max rel jacobian err {np.max(jerr / np.maximum(rowmax[rows], 1e-300)):.3e}"
    return rowscale


def rel_err(a, b):
    a = np.asarray(a).ravel(order="F")
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def test_config1_nlpoisson_65(vfvm, oracle):
    g = grid(vfvm, 65, 2)
    assert g.nnodes == 4225
    sys = vfvm.System(g, vfvm.Physics("nlpoisson"))
    osys = oracle.OracleSystem(g, "nlpoisson")
    U = np.random.default_rng(11).uniform(-0.5, 1.0, size=(1, g.nnodes))
    Fo, Jo = osys.assemble(U.ravel(), keep_pattern=True)
    F, J = vfvm.evaluate_residual_and_jacobian(sys, U)
    check_assembly(J, F.ravel(order="F"), Jo, Fo, U.ravel())
    # the full Newton solve from u = 0, with the reference's default control
    Us = vfvm.solve(sys, inival=0.0, control=vfvm.SolverControl(maxiters_linear=400))
    uo, _ = oracle.solve_step(osys, np.zeros(g.nnodes), oracle.Control())
    assert rel_err(Us, uo) <= SOL_TOL


def mixed_residual(vfvm, sys, U, Uold, t, tstep):
    """F of the mixed form (FP64 residual, FP32 Jacobian) through the device entry point."""
    import torch
    lib = vfvm._lib.load()
    Ud = torch.from_numpy(np.ascontiguousarray(U)).cuda()
    Uod = torch.from_numpy(np.ascontiguousarray(Uold)).cuda()
    Fd = torch.empty_like(Ud)
    torch.cuda.synchronize()
    rc = lib.vfvm_assemble_device(sys.ctx, ctypes.c_void_p(Ud.data_ptr()), ctypes.c_void_p(Uod.data_ptr()), t, tstep,
                                  0.0, ctypes.c_void_p(Fd.data_ptr()), 1)
    assert rc == 0
    torch.cuda.synchronize()
    return Fd.cpu().numpy()


def test_config2_porous_513_assembly(vfvm, oracle):
    pytest.importorskip("torch")
    g = grid(vfvm, 513, 2)
    assert g.nnodes == 263169
    sys = vfvm.System(g, vfvm.Physics("porous"))
    osys = oracle.OracleSystem(g, "porous")
    rng = np.random.default_rng(12)
    U = rng.uniform(1e-3, 1.0, size=g.nnodes)
    Uold = rng.uniform(1e-3, 1.0, size=g.nnodes)
    Fo, Jo = osys.assemble(U, Uold, 0.0, 1e-3, 0.0, keep_pattern=True)
    F, J = vfvm.evaluate_residual_and_jacobian(sys, U.reshape(1, -1), t=0.0, tstep=1e-3, uold=Uold.reshape(1, -1))
    rowscale = check_assembly(J, F.ravel(order="F"), Jo, Fo, U)
    Fm = mixed_residual(vfvm, sys, U, Uold, 0.0, 1e-3)
    assert np.all(np.abs(Fm - Fo) <= TOL * rowscale + 1e-300)


def test_config2_porous_513_two_steps(vfvm, oracle):
    g = grid(vfvm, 513, 2)
    x, y = g.coord
    u0 = 1e-3 + np.exp(-((x - 0.5) ** 2 + (y - 0.5) ** 2) / 0.1 ** 2)
    sys = vfvm.System(g, vfvm.Physics("porous"))
    # the reference's default Newton control (update norm <= 1e-10) on both sides
    control = vfvm.fixed_timesteps(vfvm.SolverControl(precision="mixed", engine="graph", maxiters_linear=200), 1e-3)
    tsol = vfvm.solve(sys, inival=u0.reshape(1, -1), times=[0.0, 0.002], control=control)
    osys = oracle.OracleSystem(g, "porous")
    oc = oracle.fixed_timesteps(oracle.Control(), 1e-3)
    _, osols, _ = oracle.solve_transient(osys, u0, [0.0, 0.002], oc)
    assert len(tsol.u) == len(osols) == 3
    for k in (1, 2):
        assert rel_err(tsol.u[k], osols[k]) <= SOL_TOL


def test_config3_bipolar_64cubed_assembly(vfvm, oracle):
    g = grid(vfvm, 64, 3)
    assert g.nnodes == 262144
    sys = vfvm.System(g, vfvm.Physics("bipolar", BIPOLAR), species=[1, 2, 3])
    osys = oracle.OracleSystem(g, "bipolar", BIPOLAR)
    rng = np.random.default_rng(13)
    U = np.empty((3, g.nnodes))
    U[0] = rng.uniform(-1.0, 1.0, size=g.nnodes)
    U[1] = rng.uniform(0.5, 2.0, size=g.nnodes)
    U[2] = rng.uniform(0.5, 2.0, size=g.nnodes)
    U = np.asfortranarray(U)
    u = U.ravel(order="F")
    Fo, Jo = osys.assemble(u, u, 0.0, np.inf, 0.5, keep_pattern=True)
    F, J = vfvm.evaluate_residual_and_jacobian(sys, U, embed=0.5)
    check_assembly(J, F.ravel(order="F"), Jo, Fo, u)


def test_config4_rd2_batch_largest_side(vfvm, oracle):
    pytest.importorskip("torch")
    import torch
    sides = (257, 33, 101)
    prm = [(0.3, 2.5, 1.7), (5.0, 0.05, 20.0), (0.02, 0.8, 0.1)]
    grids = [grid(vfvm, m, 2) for m in sides]
    systems = [vfvm.System(gr, vfvm.Physics("rd2", list(p)), species=[1, 2]) for gr, p in zip(grids, prm)]
    batch = vfvm.BatchSolver(systems)
    U0 = torch.full((batch.ndofs,), 0.5, dtype=torch.float64, device="cuda")
    U = torch.empty_like(U0)
    c = vfvm.SolverControl(precision="mixed", precon_linear="ilu0", coarse=100, maxiters_linear=1000)
    hist = batch.solve_device(U0.data_ptr(), U.data_ptr(), c)
    assert all(h.status == 0 for h in hist)
    off = batch.offsets
    Uh = U.cpu().numpy()
    oc = oracle.Control()  # the reference's default Newton control on both sides
    for i, (gr, p) in enumerate(zip(grids, prm)):
        osys = oracle.OracleSystem(gr, "rd2", list(p))
        uo, _ = oracle.solve_step(osys, np.full(2 * gr.nnodes, 0.5), oc)
        assert rel_err(Uh[off[i]:off[i + 1]], uo) <= SOL_TOL, f"instance {i} (side {sides[i]})"
