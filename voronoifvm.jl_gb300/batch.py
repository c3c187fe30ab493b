"""Batched solves of many systems of one physics (uneven grids and parameters).

The reference runs such sweeps as one ``SystemState`` per thread
(``examples/Example440_ParallelState.jl:36-45``).  Here all systems are solved
together in one persistent cooperative launch on the GPU: a group of CTAs per
system, largest systems first, the number of CTAs per system chosen by the
autotuner (``tune``)."""
from __future__ import annotations

import ctypes
import math
from typing import List, Optional, Sequence

import numpy as np

from . import _lib as L
from .system import NewtonSolverHistory, SolverControl, System, _flat, _raise, _shape


def _check_f64_device(t):
    if not (getattr(t, "is_cuda", False) and str(t.dtype) == "torch.float64" and t.is_contiguous()):
        raise ValueError("expected a contiguous float64 CUDA tensor")

__all__ = ["BatchSolver"]


class BatchSolver:
    def __init__(self, systems: Sequence[System]):
        if not systems:
            raise ValueError("empty batch")
        kinds = {s.physics.kind for s in systems}
        if len(kinds) != 1:
            raise ValueError(f"a batch holds one physics kind, got {sorted(kinds)}")
        lib = L.load()
        self.systems = list(systems)
        # systems built on one Grid object pass the same grid arrays, so the
        # library keeps a single copy of the grid tables for them
        marshalled, first = [], {}
        for s in self.systems:
            gt, pt, keep = s._marshal()
            gt = first.setdefault(id(s.grid), gt)
            marshalled.append((gt, pt, keep))
        self._keep = [m[2] for m in marshalled]
        n = len(self.systems)
        grids = (L.Grid_t * n)(*[m[0] for m in marshalled])
        phys = (L.Physics_t * n)(*[m[1] for m in marshalled])
        status = ctypes.c_int(0)
        self.h = lib.vfvm_batch_create(n, grids, phys, ctypes.byref(status))
        if not self.h:
            _raise(status.value or L.ERR_INPUT, "vfvm_batch_create failed")
        self.offsets = np.zeros(n + 1, dtype=np.int64)
        _raise(lib.vfvm_batch_offsets(self.h, L.ptr(self.offsets, L.c_i64)))
        self.history: List[NewtonSolverHistory] = []
        self.best_ctas: Optional[int] = None

    def _info(self):
        out = np.zeros(7, dtype=np.int64)
        _raise(L.load().vfvm_batch_info(self.h, L.ptr(out, L.c_i64)), "vfvm_batch_info")
        return out

    @property
    def graphed(self) -> bool:
        """True if the last solve ran as a captured CUDA graph."""
        return bool(self._info()[3])

    @property
    def launches(self) -> int:
        """Kernels launched by the last solve."""
        return int(self._info()[6])

    @property
    def engine(self) -> str:
        """Engine of the last solve: "persistent" (CTA teams) or "sweep" (whole-GPU kernels)."""
        return "sweep" if self._info()[4] == 1 else "persistent"

    @property
    def ninst(self) -> int:
        return len(self.systems)

    @property
    def ndofs(self) -> int:
        return int(self.offsets[-1])

    def pack(self, inivals) -> np.ndarray:
        out = np.empty(self.ndofs)
        for i, (s, u) in enumerate(zip(self.systems, inivals)):
            out[self.offsets[i]:self.offsets[i + 1]] = _flat(u, s)
        return out

    def unpack(self, U: np.ndarray):
        return [_shape(U[self.offsets[i]:self.offsets[i + 1]].copy(), s) for i, s in enumerate(self.systems)]

    def set_instance(self, i: int, data=None, nodedata=None):
        """Replace the parameters and/or node data of instance i (same sizes)."""
        s = self.systems[i]
        if data is not None:
            s.physics.data = list(np.atleast_1d(np.asarray(data, dtype=np.float64)))
        p = np.ascontiguousarray(s.physics.data, dtype=np.float64)
        nd, ndp = 0, None
        if nodedata is not None:
            a = np.asarray(nodedata, dtype=np.float64)
            a = a.reshape(-1, s.grid.nnodes) if a.ndim == 1 else a
            s.physics.nodedata = a
            nda = np.ascontiguousarray(a.T)
            nd, ndp = a.shape[0], L.ptr(nda)
        _raise(L.load().vfvm_batch_set_instance(self.h, i, L.ptr(p), p.size, ndp, nd), "vfvm_batch_set_instance")

    def load_device(self, params=None, nodedata=None):
        """Replace every system's parameters and/or node data from device tensors:
        ``params`` (ninst, nparams) float64, ``nodedata`` the systems' (nnodes_i,
        nnodedata) node-major blocks packed in system order (for one shared grid:
        (ninst, nnodes) when nnodedata == 1).  No host copies; the Python-side
        ``physics`` records of the systems are not updated."""
        pp, npar, nd, nnd = None, 0, None, 0
        if params is not None:
            _check_f64_device(params)
            pp, npar = ctypes.c_void_p(params.data_ptr()), int(params.shape[-1]) if params.dim() > 1 else 1
        if nodedata is not None:
            _check_f64_device(nodedata)
            total = sum(s.grid.nnodes for s in self.systems)
            nd, nnd = ctypes.c_void_p(nodedata.data_ptr()), nodedata.numel() // total
        _raise(L.load().vfvm_batch_load_device(self.h, pp, npar, nd, nnd), "vfvm_batch_load_device")

    def _control(self, control):
        c = (control or SolverControl()).to_c(False)
        if self.best_ctas and c.team_ctas == 0:
            c.team_ctas = self.best_ctas
        return c

    def solve(self, inivals, control: Optional[SolverControl] = None, time: float = 0.0, tstep: float = math.inf,
              embed: float = 0.0, check: bool = True):
        """Solve every system from its initial value; returns the list of solutions."""
        lib = L.load()
        U0 = self.pack(inivals)
        U = np.zeros_like(U0)
        hist = (L.History_t * self.ninst)()
        c = self._control(control)
        rc = lib.vfvm_batch_solve(self.h, ctypes.byref(c), L.ptr(U0), L.ptr(U), time, tstep, embed, hist)
        self.history = [NewtonSolverHistory.from_c(h) for h in hist]
        self.status = [h.status for h in hist]
        if check:
            _raise(rc, "vfvm_batch_solve")
        return self.unpack(U)

    def solve_device(self, inival_dev: int, U_dev: int, control: Optional[SolverControl] = None, time: float = 0.0,
                     tstep: float = math.inf, embed: float = 0.0):
        """Device-resident variant: pointers to packed device arrays of ndofs doubles."""
        lib = L.load()
        hist = (L.History_t * self.ninst)()
        c = self._control(control)
        rc = lib.vfvm_batch_solve_device(self.h, ctypes.byref(c), ctypes.c_void_p(inival_dev), ctypes.c_void_p(U_dev),
                                         time, tstep, embed, hist)
        self.history = [NewtonSolverHistory.from_c(h) for h in hist]
        _raise(rc, "vfvm_batch_solve_device")
        return self.history

    def tune(self, inival_dev: int, control: Optional[SolverControl] = None, candidates=(1, 2, 4, 8)):
        """Autotune the CTAs per system on this batch (device-resident inival)."""
        lib = L.load()
        cand = np.ascontiguousarray(candidates, dtype=np.int32)
        times = np.zeros(cand.size, dtype=np.float32)
        best = ctypes.c_int32(0)
        c = (control or SolverControl()).to_c(False)
        _raise(lib.vfvm_batch_tune(self.h, ctypes.byref(c), ctypes.c_void_p(inival_dev), ctypes.byref(best),
                                   times.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), cand.size,
                                   L.ptr(cand, L.c_i32)), "vfvm_batch_tune")
        self.best_ctas = int(best.value)
        return self.best_ctas, dict(zip(cand.tolist(), times.tolist()))

    def close(self):
        if getattr(self, "h", None):
            L.load().vfvm_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
