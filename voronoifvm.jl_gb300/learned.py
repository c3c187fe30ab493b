"""Learned Newton initial iterate for many solves of one parametrised problem.

Workload: stationary ``-div(kappa grad u) + exp(u) = f`` on the unit square
(triangles from ``simplexgrid``), ``u = 0`` on the whole boundary, with
``kappa = exp(G)``, ``G`` a Gaussian random field and ``f`` one scalar per
instance (the ``kappa_exp`` physics).

Pipeline (no counterpart in the reference, whose ``solve`` always starts from
``inival``, ``src/vfvm_solver.jl:551-668``):

* ``grf_logkappa`` samples ``G`` with covariance ``sigma^2 exp(-r^2/(2 ell^2))``
  by a truncated Fourier series on a periodic square of side 2 (so that the
  unit square sees no wrap-around correlation), seeded per instance;
* ``KappaSweep`` solves many instances on one shared grid with the batched
  device solver (training data, and the evaluation itself);
* ``Network`` is the device multilayer perceptron of the C ABI (BF16 operands,
  FP32 accumulation, forward/backward/Adam kernels of this library);
* ``LearnedInitialIterate`` maps (G on a coarse nc x nc subgrid, f) to the
  solution on the same coarse subgrid, prolongs it bilinearly to the fine grid
  on the device and hands it to the guarded batched solve: Newton runs from the
  prediction while every iteration reduces the FP64 residual and restarts from
  the user's ``inival`` where one does not (or Newton fails otherwise).
"""
from __future__ import annotations

import ctypes
import math
from typing import Optional, Sequence

import numpy as np

from . import _lib as L
from .batch import BatchSolver
from .grid import simplexgrid
from .system import NewtonSolverHistory, Physics, SolverControl, System, _raise

__all__ = ["grf_logkappa", "kappa_instance", "kappa_scale", "mesh_symmetries", "Network", "KappaSweep",
           "LearnedInitialIterate"]


def grf_logkappa(n: int, seed: int, ell: float = 0.1, sigma: float = 1.0, modes: int = 20,
                 period: float = 2.0) -> np.ndarray:
    """Gaussian random field on the n x n nodes of the unit square (node order
    ix + n*iy), covariance sigma^2 exp(-r^2 / (2 ell^2)), seeded.

    Fourier series on a periodic square of side ``period`` with wave numbers
    k = m / period, |m_x|, |m_y| <= modes; each mode carries independent N(0,1)
    cosine and sine amplitudes scaled by sqrt(S(k)) / period, S the spectral
    density sigma^2 2 pi ell^2 exp(-2 pi^2 ell^2 |k|^2).  With ell = 0.1 the
    omitted modes carry less than 1e-8 of the variance."""
    rng = np.random.default_rng([int(seed), 0x6B617070])
    m = np.arange(-modes, modes + 1)
    k = m / period
    K2 = k[:, None] ** 2 + k[None, :] ** 2
    S = sigma ** 2 * 2.0 * math.pi * ell ** 2 * np.exp(-2.0 * math.pi ** 2 * ell ** 2 * K2)
    amp = np.sqrt(S) / period
    A = rng.standard_normal(amp.shape) * amp
    B = rng.standard_normal(amp.shape) * amp
    x = np.linspace(0.0, 1.0, n)
    ph = 2.0 * math.pi * np.outer(x, k)
    C, Sn = np.cos(ph), np.sin(ph)
    # G[ix, iy] = sum_m amp (a cos(kx x + ky y) + b sin(kx x + ky y))
    G = C @ A @ C.T - Sn @ A @ Sn.T + Sn @ B @ C.T + C @ B @ Sn.T
    return np.ascontiguousarray(G.T).ravel()


def kappa_scale(f) -> np.ndarray:
    """Per-instance output factor of the kappa_exp surrogate: f - 1.  Linearised
    at u = 0 the problem reads -div(kappa grad u) + u = f - 1, so u / (f - 1) is
    nearly independent of f and the network learns that ratio (kept away from
    0 by 1e-3 for f close to 1)."""
    s = np.asarray(f, dtype=np.float64) - 1.0
    return np.where(np.abs(s) < 1e-3, np.copysign(1e-3, s), s)


def kappa_instance(n: int, seed: int, ell: float = 0.1, sigma: float = 1.0):
    """(log kappa on the n x n nodes, f uniform in [-1, 1]) of instance ``seed``."""
    G = grf_logkappa(n, seed, ell, sigma)
    f = float(np.random.default_rng([int(seed), 0x66]).uniform(-1.0, 1.0))
    return G, f


def mesh_symmetries(a: np.ndarray, m: int):
    """The four images of node fields on an m x m square grid (rows of ``a``,
    node order ix + m*iy) under the symmetries of the triangulation: identity,
    rotation by 180 degrees, reflection across the diagonal x = y and across
    x = 1 - y.  simplexgrid splits every square along its (0,0)-(1,1)
    diagonal, which these four maps (and not the rotations by 90 degrees)
    preserve, so the discrete kappa_exp problem -- u = 0 on the whole boundary,
    isotropic kappa -- maps each solution onto the solution of the mapped
    coefficient field exactly.  Returns an array of shape (4, S, m*m)."""
    A = np.asarray(a).reshape(-1, m, m)  # [s, iy, ix]
    T = A.transpose(0, 2, 1)
    return np.stack([A, A[:, ::-1, ::-1], T, T[:, ::-1, ::-1]]).reshape(4, A.shape[0], m * m)


class Network:
    """The device multilayer perceptron (vfvm_mlp_* of the C ABI).

    ``sizes``: inputs, hidden widths..., outputs.  Inputs/targets are CUDA
    float32 torch tensors of shape (batch, sizes[0]) / (batch, sizes[-1])."""

    def __init__(self, sizes: Sequence[int], max_batch: int, seed: int = 0):
        self.sizes = [int(s) for s in sizes]
        self.max_batch = int(max_batch)
        arr = (ctypes.c_int32 * len(self.sizes))(*self.sizes)
        st = ctypes.c_int(0)
        self.h = L.load().vfvm_mlp_create(len(self.sizes) - 1, arr, self.max_batch, seed, ctypes.byref(st))
        if not self.h:
            _raise(st.value or L.ERR_INPUT, "vfvm_mlp_create")

    @property
    def nparams(self) -> int:
        n = ctypes.c_int64(0)
        _raise(L.load().vfvm_mlp_nparams(self.h, ctypes.byref(n)))
        return int(n.value)

    def get_params(self) -> np.ndarray:
        out = np.empty(self.nparams, dtype=np.float32)
        _raise(L.load().vfvm_mlp_params(self.h, L.ptr(out, ctypes.c_float), None), "vfvm_mlp_params")
        return out

    def set_params(self, theta: np.ndarray):
        t = np.ascontiguousarray(theta, dtype=np.float32)
        if t.size != self.nparams:
            raise ValueError("parameter vector has the wrong size")
        _raise(L.load().vfvm_mlp_params(self.h, None, L.ptr(t, ctypes.c_float)), "vfvm_mlp_params")

    def _check(self, X, ncols):
        import torch
        if not (X.is_cuda and X.dtype == torch.float32 and X.is_contiguous() and X.dim() == 2
                and X.shape[1] == ncols and 1 <= X.shape[0] <= self.max_batch):
            raise ValueError(f"expected a contiguous CUDA float32 tensor (b <= {self.max_batch}, {ncols})")

    def forward(self, X):
        import torch
        self._check(X, self.sizes[0])
        Y = torch.empty((X.shape[0], self.sizes[-1]), dtype=torch.float32, device=X.device)
        _raise(L.load().vfvm_mlp_forward(self.h, X.shape[0], X.data_ptr(), Y.data_ptr()), "vfvm_mlp_forward")
        return Y

    def gradients(self, X, T):
        """(loss, flat gradient in get_params order) of the mean squared error."""
        self._check(X, self.sizes[0])
        self._check(T, self.sizes[-1])
        g = np.empty(self.nparams, dtype=np.float32)
        loss = ctypes.c_float(0)
        _raise(L.load().vfvm_mlp_gradients(self.h, X.shape[0], X.data_ptr(), T.data_ptr(), L.ptr(g, ctypes.c_float),
                                           ctypes.byref(loss)), "vfvm_mlp_gradients")
        return float(loss.value), g

    def train_step(self, X, T, lr: float, want_loss: bool = False) -> Optional[float]:
        loss = ctypes.c_float(0)
        _raise(L.load().vfvm_mlp_train_step(self.h, X.shape[0], X.data_ptr(), T.data_ptr(), float(lr),
                                            ctypes.byref(loss) if want_loss else None), "vfvm_mlp_train_step")
        return float(loss.value) if want_loss else None

    def close(self):
        if getattr(self, "h", None):
            L.load().vfvm_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class KappaSweep:
    """``batch`` instances of the kappa_exp problem on one shared n x n grid,
    solved together by the batched device solver; instances are replaced with
    ``load`` between solves."""

    def __init__(self, n: int, batch: int):
        self.n = int(n)
        x = np.linspace(0.0, 1.0, self.n)
        self.grid = simplexgrid(x, x)
        ones = np.ones(self.grid.nnodes)
        self.systems = [System(self.grid, Physics("kappa_exp", [0.0], ones)) for _ in range(batch)]
        self.solver = BatchSolver(self.systems)
        self.nnodes = self.grid.nnodes

    @property
    def batch(self) -> int:
        return len(self.systems)

    def load(self, logk: np.ndarray, f: np.ndarray):
        """Instance i gets kappa = exp(logk[i]) and source f[i] (i < len(f))."""
        for i in range(len(f)):
            self.solver.set_instance(i, data=[float(f[i])], nodedata=np.exp(logk[i]))

    def load_device(self, kappa, f):
        """All instances at once from device tensors: kappa (batch, nnodes) and
        f (batch,), both float64."""
        self.solver.load_device(params=f.reshape(-1, 1), nodedata=kappa)

    def solve_device(self, inival_dev: int, U_dev: int, control: SolverControl, guess_dev: Optional[int] = None):
        """Solve all instances (packed device arrays of batch * nnodes doubles);
        with guess_dev, the guarded start.  Returns (histories, from_guess)."""
        if guess_dev is None:
            return self.solver.solve_device(inival_dev, U_dev, control), np.zeros(self.batch, dtype=np.int32)
        s = self.solver
        hist = (L.History_t * s.ninst)()
        fg = np.zeros(s.ninst, dtype=np.int32)
        c = s._control(control)
        rc = L.load().vfvm_batch_solve_guarded_device(s.h, ctypes.byref(c), ctypes.c_void_p(guess_dev),
                                                      ctypes.c_void_p(inival_dev), ctypes.c_void_p(U_dev), 0.0,
                                                      math.inf, 0.0, hist, L.ptr(fg, L.c_i32))
        s.history = [NewtonSolverHistory.from_c(h) for h in hist]
        _raise(rc, "vfvm_batch_solve_guarded_device")
        return s.history, fg

    def close(self):
        self.solver.close()


class LearnedInitialIterate:
    """Coarse-grid surrogate of the kappa_exp solution map (G, f) -> u.

    Features: G at the nodes of the nc x nc subgrid (every r-th fine node,
    n = (nc-1) r + 1), or with ``half`` > 0 its mean over the (2 half + 1)^2
    fine nodes around each of them, and f; targets: u at the subgrid nodes,
    standardised with the training mean and standard deviation.  ``layers``
    linear layers of width ``hidden`` (ReLU between)."""

    def __init__(self, n: int, nc: int, hidden: int = 512, layers: int = 4, max_batch: int = 512, seed: int = 0,
                 half: int = 0):
        if (n - 1) % (nc - 1):
            raise ValueError("the coarse grid must nest in the fine grid: (n-1) % (nc-1) == 0")
        self.n, self.nc, self.r = n, nc, (n - 1) // (nc - 1)
        if not 0 <= half <= self.r:
            raise ValueError("the feature window half-width must lie in [0, (n-1)/(nc-1)]")
        self.half = int(half)
        self.sizes = [nc * nc + 1] + [hidden] * (layers - 1) + [nc * nc]
        self.net = Network(self.sizes, max_batch, seed)
        self.mean, self.std = 0.0, 1.0

    def coarse(self, fine: np.ndarray) -> np.ndarray:
        """Values at the coarse subgrid nodes of (S, n*n) fine node arrays."""
        F = np.asarray(fine).reshape(-1, self.n, self.n)  # [iy, ix]
        return F[:, ::self.r, ::self.r].reshape(F.shape[0], -1)

    def augment(self, X: np.ndarray, T: np.ndarray, scale=None):
        """Training pairs under the mesh symmetries (mesh_symmetries): features X
        (S, nc*nc + 1: coarse field, then f) and coarse targets T (S, nc*nc)
        become 4 S pairs; `scale` (S,) is repeated alongside."""
        nc2 = self.nc * self.nc
        Xs = mesh_symmetries(X[:, :nc2], self.nc)
        fcol = np.broadcast_to(X[:, nc2:], (4,) + X[:, nc2:].shape)
        Xa = np.concatenate([Xs, fcol], axis=2).reshape(-1, X.shape[1]).astype(X.dtype)
        Ta = mesh_symmetries(T, self.nc).reshape(-1, nc2)
        Sa = None if scale is None else np.tile(np.asarray(scale), 4)
        return Xa, Ta, Sa

    def coarse_mean(self, fine: np.ndarray) -> np.ndarray:
        """Means of (S, n*n) fine node arrays over the (2 half + 1)^2 window
        around each coarse subgrid node (clipped at the boundary)."""
        n, h = self.n, self.half
        F = np.asarray(fine, dtype=np.float64).reshape(-1, n, n)
        C = np.zeros((F.shape[0], n + 1, n + 1))
        C[:, 1:, 1:] = F.cumsum(1).cumsum(2)
        c = np.arange(self.nc) * self.r
        lo, hi = np.clip(c - h, 0, n - 1), np.clip(c + h, 0, n - 1) + 1
        S = C[:, hi][:, :, hi] - C[:, lo][:, :, hi] - C[:, hi][:, :, lo] + C[:, lo][:, :, lo]
        return (S / ((hi - lo)[:, None] * (hi - lo)[None, :])).reshape(F.shape[0], -1)

    def features(self, logk: np.ndarray, f: np.ndarray) -> np.ndarray:
        G = self.coarse(logk) if self.half == 0 else self.coarse_mean(logk)
        return np.ascontiguousarray(np.concatenate([G, np.asarray(f).reshape(-1, 1)], axis=1), dtype=np.float32)

    def features_from_kappa(self, kappa: np.ndarray, f: np.ndarray) -> np.ndarray:
        """The same features from the node data kappa = exp(G), on the host."""
        G = np.log(self.coarse(kappa)) if self.half == 0 else self.coarse_mean(np.log(kappa))
        return np.ascontiguousarray(np.concatenate([G, np.asarray(f).reshape(-1, 1)], axis=1), dtype=np.float32)

    def features_device(self, kappa_d, f_d, out=None):
        """The same features on the device from kappa = exp(G) (CUDA float64,
        S x n*n) and f (CUDA float64, S values): CUDA float32, S x (nc*nc + 1)."""
        import torch
        S = f_d.numel()
        if not (kappa_d.is_cuda and kappa_d.dtype == torch.float64 and kappa_d.is_contiguous()
                and kappa_d.numel() == S * self.n * self.n and f_d.dtype == torch.float64 and f_d.is_contiguous()):
            raise ValueError("kappa: contiguous CUDA float64 S x n*n; f: contiguous CUDA float64, S values")
        nin = self.nc * self.nc + 1
        if out is None:
            out = torch.empty((S, nin), dtype=torch.float32, device=kappa_d.device)
        _raise(L.load().vfvm_coarse_log_features(S, self.nc, self.r, self.half, kappa_d.data_ptr(), self.n * self.n,
                                                 f_d.data_ptr(), out.data_ptr(), None), "vfvm_coarse_log_features")
        return out

    def fit(self, X: np.ndarray, U: np.ndarray, scale=None, epochs: int = 200, batch: int = 256, lr: float = 1e-3,
            lr_final: float = 1e-5, seed: int = 0, log_every: int = 0):
        """Train on features X (S, nin) and solutions U: fine (S, n*n) or already
        restricted to the coarse subgrid (S, nc*nc).  With `scale` (S,), the
        network learns U / scale (see kappa_scale) and predict_device multiplies
        back.  Adam with a cosine learning-rate decay.  Returns the per-epoch
        training losses."""
        import torch
        U = np.asarray(U)
        T = U if U.shape[1] == self.nc * self.nc else self.coarse(U)
        if scale is not None:
            T = T / np.asarray(scale, dtype=np.float64)[:, None]
        self.mean, self.std = float(T.mean()), float(T.std() + 1e-30)
        dev = torch.device("cuda")
        Xd = torch.from_numpy(np.ascontiguousarray(X, dtype=np.float32)).to(dev)
        Td = torch.from_numpy(((T - self.mean) / self.std).astype(np.float32)).to(dev)
        S = Xd.shape[0]
        batch = min(batch, self.net.max_batch, S)
        rng = np.random.default_rng(seed)
        steps_per_epoch = max(1, S // batch)
        total = epochs * steps_per_epoch
        losses, step = [], 0
        for ep in range(epochs):
            perm = torch.from_numpy(rng.permutation(S)).to(dev)
            for j in range(steps_per_epoch):
                idx = perm[j * batch:(j + 1) * batch]
                xb, tb = Xd[idx].contiguous(), Td[idx].contiguous()
                a = lr_final + 0.5 * (lr - lr_final) * (1.0 + math.cos(math.pi * step / max(1, total - 1)))
                last = j + 1 == steps_per_epoch
                l = self.net.train_step(xb, tb, a, want_loss=last)
                step += 1
            losses.append(l)
            if log_every and (ep % log_every == 0 or ep + 1 == epochs):
                print(f"epoch {ep}: loss {l:.3e}")
        return losses

    def predict_coarse(self, Xd):
        """Standardised coarse solution prediction (CUDA float32, S x nc*nc)."""
        return self.net.forward(Xd)

    def predict_device(self, Xd, scale=None, out=None):
        """Fine initial values (CUDA float64, S x n*n) for features Xd on the
        device; `scale`: the per-instance factors used in fit (CUDA float64
        tensor of S values), or None."""
        import torch
        Yc = self.predict_coarse(Xd).contiguous()
        S = Yc.shape[0]
        if out is None:
            out = torch.empty((S, self.n * self.n), dtype=torch.float64, device=Xd.device)
        sp = None
        if scale is not None:
            if not (scale.is_cuda and scale.dtype == torch.float64 and scale.numel() == S and scale.is_contiguous()):
                raise ValueError("scale must be a contiguous CUDA float64 tensor with one value per instance")
            sp = scale.data_ptr()
        _raise(L.load().vfvm_prolong_bilinear(S, self.nc, self.r, Yc.data_ptr(), self.nc * self.nc, self.std,
                                              self.mean, sp, out.data_ptr(), self.n * self.n, None),
               "vfvm_prolong_bilinear")
        return out

    def close(self):
        self.net.close()
