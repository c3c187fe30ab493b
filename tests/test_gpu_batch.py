"""Batched solves (one persistent launch for many systems of uneven size)."""
import json
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN
from gpu_cases import lin

pytestmark = pytest.mark.gpu
RTOL = math.sqrt(np.finfo(float).eps)


def test_example440_as_one_batch(vfvm):
    # examples/Example440_ParallelState.jl: 100 data values, one system each; the
    # reference runs one SystemState per thread, here all 100 solve in one launch
    with open(os.path.join(GOLDEN, "reference_testvals.json")) as f:
        testval = json.load(f)["Example440_ParallelState"]["value"]
    g = vfvm.simplexgrid(np.array([i / 320 for i in range(321)]))
    systems = [vfvm.System(g, vfvm.Physics("ex440", [i * 10.0 / 99.0])) for i in range(100)]
    batch = vfvm.BatchSolver(systems)
    control = vfvm.SolverControl(abstol=1e-15, reltol=1e-20, reltol_linear=1e-12, maxiters_linear=1000)
    sols = batch.solve([np.full(321, 0.1)] * 100, control=control)
    assert batch.graphed  # one captured graph: scheduler resets + the persistent launch
    total = sum(float(vfvm.integrate(s, u)[0]) for s, u in zip(systems, sols))
    assert total == pytest.approx(testval, rel=RTOL)


@pytest.mark.parametrize("coarse", [0, 60])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("precon", ["jacobi", "ilu0", "block_ilu0"])
def test_rd2_batch_vs_oracle(vfvm, oracle, precision, precon, coarse):
    rng = np.random.default_rng(7)
    sizes = [9, 25, 13, 17, 21, 11]
    systems, params = [], []
    for n in sizes:
        p = list(10.0 ** rng.uniform(-1, 1, size=3))
        params.append(p)
        systems.append(vfvm.System(vfvm.simplexgrid(lin(n - 1), lin(n - 1)), vfvm.Physics("rd2", p), species=[1, 2]))
    batch = vfvm.BatchSolver(systems)
    control = vfvm.SolverControl(precision=precision, precon_linear=precon, maxiters_linear=500, coarse=coarse)
    sols = batch.solve([np.full(s.ndofs, 0.5) for s in systems], control=control)
    for s, p, u in zip(systems, params, sols):
        osys = oracle.OracleSystem(s.grid, "rd2", p)
        uo, _ = oracle.solve_step(osys, np.full(osys.n, 0.5), oracle.Control())
        err = np.max(np.abs(u.ravel(order="F") - uo)) / np.max(np.abs(uo))
        assert err <= 1e-8


def test_batch_tune(vfvm):
    torch = pytest.importorskip("torch")
    systems = [vfvm.System(vfvm.simplexgrid(lin(n), lin(n)), vfvm.Physics("nlpoisson")) for n in (8, 16, 24, 32)]
    batch = vfvm.BatchSolver(systems)
    u0 = torch.zeros(batch.ndofs, dtype=torch.float64, device="cuda")
    best, times = batch.tune(u0.data_ptr(), candidates=(1, 2, 4))
    assert best in (1, 2, 4)
    assert all(t > 0 for t in times.values())
    sols = batch.solve([np.zeros(s.ndofs) for s in systems])
    ref = vfvm.solve(systems[-1], inival=0.0)
    assert np.max(np.abs(sols[-1] - ref)) <= 1e-8 * np.max(np.abs(ref))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_sweep_engine_matches_cta_teams(vfvm, oracle, precision):
    # a shared-grid batch runs on the sweep engine (whole-GPU kernels over all
    # systems); the same batch on the CTA-team engine and the oracle agree with it
    import torch
    g = vfvm.simplexgrid(lin(24), lin(24))
    rng = np.random.default_rng(11)
    kappas = [np.exp(rng.normal(size=g.nnodes)) for _ in range(5)]
    fs = [-0.9, -0.2, 0.3, 0.8, 0.0]
    systems = [vfvm.System(g, vfvm.Physics("kappa_exp", [f], k)) for f, k in zip(fs, kappas)]
    batch = vfvm.BatchSolver(systems)
    U0 = torch.zeros(batch.ndofs, dtype=torch.float64, device="cuda")
    out = {}
    for engine in ("auto", "persistent"):
        c = vfvm.SolverControl(precision=precision, coarse=50, engine=engine, updatecontrol=False, abstol=1e-12,
                               reltol=0.0, maxiters_linear=500)
        U = torch.empty_like(U0)
        hist = batch.solve_device(U0.data_ptr(), U.data_ptr(), c)
        assert all(h.status == 0 for h in hist)
        out[batch.engine] = U.cpu().numpy()
    assert set(out) == {"sweep", "persistent"}
    assert np.max(np.abs(out["sweep"] - out["persistent"])) <= 1e-9 * np.max(np.abs(out["persistent"]))
    for i, (f, k) in enumerate(zip(fs, kappas)):
        osys = oracle.OracleSystem(g, "kappa_exp", [f], nodedata=k)
        uo, _ = oracle.solve_step(osys, np.zeros(g.nnodes), oracle.Control(abstol=1e-12, reltol=1e-20))
        u = out["sweep"][batch.offsets[i]:batch.offsets[i + 1]]
        assert np.max(np.abs(u - uo)) <= 1e-8 * np.max(np.abs(uo))


@pytest.mark.parametrize("engine", ["auto", "persistent"])
def test_load_device_matches_set_instance(vfvm, engine):
    # all instances replaced from device arrays in one call give the same
    # solutions, bit for bit, as per-instance host updates; both engines
    import torch
    g = vfvm.simplexgrid(lin(20), lin(20))
    rng = np.random.default_rng(21)
    S = 6
    systems = [vfvm.System(g, vfvm.Physics("kappa_exp", [0.0], np.ones(g.nnodes))) for _ in range(S)]
    batch = vfvm.BatchSolver(systems)
    c = vfvm.SolverControl(precision="mixed", coarse=40, engine=engine, maxiters_linear=500)
    U0 = torch.zeros(batch.ndofs, dtype=torch.float64, device="cuda")
    batch.solve_device(U0.data_ptr(), torch.empty_like(U0).data_ptr(), c)  # builds the engine's state first
    runs = []
    for _ in range(2):
        kappa = np.exp(rng.normal(size=(S, g.nnodes)))
        f = rng.uniform(-1.0, 1.0, size=S)
        for i in range(S):
            batch.set_instance(i, data=[f[i]], nodedata=kappa[i])
        Ua = torch.empty_like(U0)
        batch.solve_device(U0.data_ptr(), Ua.data_ptr(), c)
        batch.load_device(params=torch.from_numpy(np.flip(f).copy()).reshape(-1, 1).cuda(),
                          nodedata=torch.from_numpy(np.flip(kappa, 0).copy()).cuda())  # other values first
        batch.load_device(params=torch.from_numpy(f).reshape(-1, 1).cuda(), nodedata=torch.from_numpy(kappa).cuda())
        Ub = torch.empty_like(U0)
        hist = batch.solve_device(U0.data_ptr(), Ub.data_ptr(), c)
        assert all(h.status == 0 for h in hist)
        assert torch.equal(Ua, Ub)
        runs.append(Ub.cpu().numpy())
    assert batch.engine == ("sweep" if engine == "auto" else "persistent")
    assert np.max(np.abs(runs[0] - runs[1])) > 0  # the second load changed the problems
    with pytest.raises(ValueError):
        batch.load_device(params=torch.zeros((S, 2), dtype=torch.float64, device="cuda"))


@pytest.mark.parametrize("tail", [0, 6, 24])
def test_sweep_batch_krylov_tail_rule(vfvm, oracle, tail):
    """The batch-level inexact Newton rule of the sweep engine: a Newton step's
    BiCGStab loop ends for all systems once at most `tail` still iterate and
    they are at most a tenth of those that entered it; those continue from
    their current iterate, and every system still meets the FP64 residual test
    and the oracle's solution (1e-8).  Tail 6 of 24 systems cuts at 2; tail
    24 cuts the late Newton steps, where only a few systems remain, never."""
    torch = pytest.importorskip("torch")
    lk = vfvm.learned
    S, n = 24, 33
    inst = [lk.kappa_instance(n, 2000 + s) for s in range(S)]
    logk = np.array([a for a, _ in inst])
    f = np.array([b for _, b in inst])
    sweep = lk.KappaSweep(n, S)
    sweep.load(logk, f)
    N = sweep.nnodes
    z = torch.zeros(S * N, dtype=torch.float64, device="cuda")
    U = torch.empty_like(z)
    control = vfvm.SolverControl(precision="mixed", coarse=40, updatecontrol=False, abstol=1e-12, reltol=0.0,
                                 maxiters_linear=50, batch_krylov_tail=tail)
    hist, _ = sweep.solve_device(z.data_ptr(), U.data_ptr(), control)
    assert sweep.solver.engine == "sweep"
    assert all(h.status == 0 for h in hist)
    Uh = U.view(S, N).cpu().numpy()
    oc = oracle.Control(abstol=1e-12, reltol=0.0)
    oc.updatecontrol = False
    for i in (0, 7, 23):
        osys = oracle.OracleSystem(sweep.grid, "kappa_exp", [f[i]], nodedata=np.exp(logk[i]))
        uo, _ = oracle.solve_step(osys, np.zeros(N), oc)
        assert np.max(np.abs(Uh[i] - uo)) <= 1e-8 * np.max(np.abs(uo))
    sweep.close()
