"""Learned initial iterate: the device network's forward pass, gradients and
Adam step against the CPU oracle, the prolongation kernel, the guarded batched
solve, and what the trained network gains over plain Newton from inival."""
import numpy as np
import pytest

import mlp_oracle as mo

pytestmark = pytest.mark.gpu

SIZES = [37, 70, 48, 20]  # deliberately not multiples of the 64-wide tiles


def _net(vfvm, seed=3, batch=50):
    import torch
    rng = np.random.default_rng(seed)
    net = vfvm.learned.Network(SIZES, max_batch=64, seed=seed)
    theta = (rng.normal(size=net.nparams) * 0.2).astype(np.float32)
    net.set_params(theta)
    X = rng.normal(size=(batch, SIZES[0])).astype(np.float32)
    T = rng.normal(size=(batch, SIZES[-1])).astype(np.float32)
    return net, theta, X, T, torch.from_numpy(X).cuda(), torch.from_numpy(T).cuda()


def test_mlp_params_roundtrip(vfvm):
    net, theta, *_ = _net(vfvm)
    assert np.array_equal(net.get_params(), theta)


def test_mlp_forward_vs_oracle(vfvm):
    net, theta, X, T, Xd, Td = _net(vfvm)
    Y = net.forward(Xd).cpu().numpy().astype(np.float64)
    Yo, _ = mo.forward(theta, SIZES, X)
    # FP32 accumulation on the device, float64 in the oracle, same bf16 operands
    assert np.linalg.norm(Y - Yo) <= 1e-3 * np.linalg.norm(Yo)


def test_mlp_gradients_vs_oracle(vfvm):
    net, theta, X, T, Xd, Td = _net(vfvm)
    loss, g = net.gradients(Xd, Td)
    lo, go = mo.loss_and_gradients(theta, SIZES, X, T)
    assert loss == pytest.approx(lo, rel=1e-4)
    assert np.linalg.norm(g - go) <= 2e-3 * np.linalg.norm(go)
    # layer by layer, so a wrong block cannot hide behind a large one
    off = 0
    for k, n in zip(SIZES[:-1], SIZES[1:]):
        for cnt in (k * n, n):
            a, b = g[off:off + cnt], go[off:off + cnt]
            assert np.linalg.norm(a - b) <= 5e-3 * np.linalg.norm(b) + 1e-9
            off += cnt


def test_mlp_adam_step_vs_oracle(vfvm):
    net, theta, X, T, Xd, Td = _net(vfvm)
    _, go = mo.loss_and_gradients(theta, SIZES, X, T)
    lr = 1e-3
    net.train_step(Xd, Td, lr)
    new = net.get_params().astype(np.float64)
    want, _, _ = mo.adam(theta.astype(np.float64), go, np.zeros_like(go), np.zeros_like(go), 1, lr)
    step, step_o = new - theta, want - theta
    # the first Adam step is about lr * sign(g): compare the steps, entries whose
    # gradient is tiny may flip sign between FP32 and float64 sums
    assert np.linalg.norm(step - step_o) <= 0.05 * np.linalg.norm(step_o)


def test_mlp_training_reduces_loss(vfvm):
    import torch
    rng = np.random.default_rng(1)
    net = vfvm.learned.Network([8, 64, 64, 4], max_batch=256, seed=0)
    X = rng.uniform(-1, 1, size=(256, 8)).astype(np.float32)
    A = rng.normal(size=(8, 4))
    T = np.tanh(X @ A).astype(np.float32)
    Xd, Td = torch.from_numpy(X).cuda(), torch.from_numpy(T).cuda()
    first = net.train_step(Xd, Td, 3e-3, want_loss=True)
    for _ in range(400):
        last = net.train_step(Xd, Td, 3e-3, want_loss=True)
    assert last < 0.05 * first


def test_prolong_bilinear(vfvm):
    import torch
    rng = np.random.default_rng(2)
    nc, r, S = 5, 4, 3
    nf = (nc - 1) * r + 1
    C = rng.normal(size=(S, nc * nc)).astype(np.float32)
    out = torch.full((S, nf * nf), np.nan, dtype=torch.float64, device="cuda")
    sc = torch.tensor([1.0, -3.0, 0.25], dtype=torch.float64, device="cuda")
    rc = vfvm._lib.load().vfvm_prolong_bilinear(S, nc, r, torch.from_numpy(C).cuda().data_ptr(), nc * nc, 2.0, 0.5,
                                                sc.data_ptr(), out.data_ptr(), nf * nf, None)
    assert rc == 0
    got = out.cpu().numpy() / sc.cpu().numpy()[:, None]
    x = np.arange(nf) / r
    for s in range(S):
        Cs = C[s].astype(np.float64).reshape(nc, nc)  # [cy, cx]
        rows = np.array([np.interp(x, np.arange(nc), Cs[j]) for j in range(nc)])  # along x
        full = np.array([np.interp(x, np.arange(nc), rows[:, i]) for i in range(nf)]).T  # along y -> [iy, ix]
        assert np.allclose(got[s].reshape(nf, nf), 2.0 * full + 0.5, rtol=0, atol=1e-12)


N_FINE, N_COARSE = 33, 9


@pytest.fixture(scope="module")
def trained(vfvm):
    """Plain solves of 192 training instances, a network trained on them, and a
    held-out set of 32 instances."""
    import torch
    lk = vfvm.learned
    ntrain, ntest = 512, 32
    sweep = lk.KappaSweep(N_FINE, ntrain)
    inst = [lk.kappa_instance(N_FINE, s) for s in range(ntrain)]
    logk = np.array([a for a, _ in inst])
    f = np.array([b for _, b in inst])
    sweep.load(logk, f)
    n = sweep.nnodes
    zeros = torch.zeros(ntrain * n, dtype=torch.float64, device="cuda")
    U = torch.empty_like(zeros)
    control = vfvm.SolverControl(updatecontrol=False, abstol=1e-10, reltol=1e-20)
    hist, _ = sweep.solve_device(zeros.data_ptr(), U.data_ptr(), control)
    assert all(h.status == 0 for h in hist)
    model = lk.LearnedInitialIterate(N_FINE, N_COARSE, hidden=256, layers=4, max_batch=256, seed=0)
    losses = model.fit(model.features(logk, f), U.cpu().numpy().reshape(ntrain, n), scale=lk.kappa_scale(f),
                       epochs=300, batch=128, lr=2e-3)
    sweep.close()
    test = [lk.kappa_instance(N_FINE, 10_000 + s) for s in range(ntest)]
    return model, losses, np.array([a for a, _ in test]), np.array([b for _, b in test])


def test_learned_gain_over_plain_newton(vfvm, oracle, trained):
    import torch
    model, losses, logk, f = trained
    assert losses[-1] < 0.05 * losses[0]
    S = len(f)
    sweep = vfvm.learned.KappaSweep(N_FINE, S)
    sweep.load(logk, f)
    n = sweep.nnodes
    control = vfvm.SolverControl(updatecontrol=False, abstol=1e-10, reltol=1e-20)
    zeros = torch.zeros(S * n, dtype=torch.float64, device="cuda")
    Up, Ul = torch.empty_like(zeros), torch.empty_like(zeros)
    hp, _ = sweep.solve_device(zeros.data_ptr(), Up.data_ptr(), control)
    X = torch.from_numpy(model.features(logk, f)).cuda()
    guess = model.predict_device(X, scale=torch.from_numpy(vfvm.learned.kappa_scale(f)).cuda())
    hl, from_guess = sweep.solve_device(zeros.data_ptr(), Ul.data_ptr(), control, guess_dev=guess.data_ptr())
    assert all(h.status == 0 for h in hp + hl)
    plain_newton = sum(h.nnewton for h in hp)
    learned_newton = sum(h.nnewton for h in hl)
    up, ul = Up.cpu().numpy().reshape(S, n), Ul.cpu().numpy().reshape(S, n)
    # the gain: on held-out instances the prediction is several times closer to the
    # solution than the user's inival (zero) ...
    pred = guess.cpu().numpy().reshape(S, n)
    err_pred = np.linalg.norm(pred - up, axis=1)
    err_inival = np.linalg.norm(up, axis=1)
    assert np.median(err_pred / err_inival) < 0.2
    # ... Newton from it succeeds for (nearly) every instance, and the held-out set
    # costs fewer Krylov iterations and no more Newton steps than from inival
    # (the work of inexact Newton grows with log(initial error / tolerance), so a
    # start several times closer saves a share of it; this problem's weak
    # nonlinearity leaves about three Newton steps either way)
    assert from_guess.sum() >= S - 2
    plain_lin = sum(h.nlin for h in hp)
    learned_lin = sum(h.nlin for h in hl)
    print(f"held-out: prediction error / inival error median {np.median(err_pred / err_inival):.3f}, "
          f"Newton steps plain {plain_newton / S:.2f}, learned {learned_newton / S:.2f}, "
          f"Krylov iterations plain {plain_lin / S:.1f}, learned {learned_lin / S:.1f}")
    assert learned_newton <= plain_newton
    assert learned_lin < plain_lin
    # both are solutions of the same problems: agree with each other and with the oracle
    # (max|F| <= 1e-10 fixes the solution of this 33 x 33 problem to about 1e-9)
    assert np.max(np.abs(up - ul)) <= 1e-8 * np.max(np.abs(up))
    g = sweep.grid
    O = oracle.OracleSystem(g, "kappa_exp", [f[0]], nodedata=np.exp(logk[0]))
    uo, _ = oracle.solve_step(O, np.zeros(n), oracle.Control(abstol=1e-12, reltol=1e-20))
    assert np.max(np.abs(ul[0] - uo)) <= 1e-8 * np.max(np.abs(uo))
    sweep.close()


def test_guarded_start_falls_back(vfvm, trained):
    import torch
    model, _, logk, f = trained
    S = 4
    sweep = vfvm.learned.KappaSweep(N_FINE, S)
    sweep.load(logk[:S], f[:S])
    n = sweep.nnodes
    control = vfvm.SolverControl(updatecontrol=False, abstol=1e-10, reltol=1e-20)
    zeros = torch.zeros(S * n, dtype=torch.float64, device="cuda")
    Up, Ug = torch.empty_like(zeros), torch.empty_like(zeros)
    hp, _ = sweep.solve_device(zeros.data_ptr(), Up.data_ptr(), control)
    guess = model.predict_device(torch.from_numpy(model.features(logk[:S], f[:S])).cuda(),
                                 scale=torch.from_numpy(vfvm.learned.kappa_scale(f[:S])).cuda()).view(-1)
    guess[:n] = float("nan")    # instance 0: a NaN guess (AssemblyError from the guess)
    guess[n:2 * n] = 1.0e3      # instance 1: exp(1000) overflows, Newton cannot reduce the residual
    hg, from_guess = sweep.solve_device(zeros.data_ptr(), Ug.data_ptr(), control, guess_dev=guess.data_ptr())
    assert from_guess.tolist() == [0, 0, 1, 1]
    assert all(h.status == 0 for h in hg)
    up, ug = Up.cpu().numpy().reshape(S, n), Ug.cpu().numpy().reshape(S, n)
    assert np.array_equal(up[:2], ug[:2])  # the fallback is plain Newton from inival
    assert np.max(np.abs(up - ug)) <= 1e-8 * np.max(np.abs(up))
    sweep.close()


@pytest.mark.parametrize("half", [0, 2])
def test_device_features_match_host(vfvm, half):
    """vfvm_coarse_log_features (log of the node data, window means around the
    coarse subgrid nodes, the source f last) equals the host features."""
    import torch
    lk = vfvm.learned
    model = lk.LearnedInitialIterate(N_FINE, N_COARSE, hidden=32, layers=2, max_batch=8, seed=0, half=half)
    inst = [lk.kappa_instance(N_FINE, 500 + s) for s in range(5)]
    logk = np.array([a for a, _ in inst])
    f = np.array([b for _, b in inst])
    Xh = model.features(logk, f)
    Xd = model.features_device(torch.from_numpy(np.exp(logk)).cuda(), torch.from_numpy(f).cuda()).cpu().numpy()
    assert Xd.shape == Xh.shape
    np.testing.assert_allclose(Xd, Xh, rtol=1e-6, atol=1e-6)
    model.close()
