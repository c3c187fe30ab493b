"""A bounded device wait that runs out returns VFVM_ERR_TIMEOUT and leaves the
CUDA context usable.

The persistent solvers' team barrier (the wait behind every grid-wide
reduction) gives up after a fixed number of polls, sets the team's error flag
and makes the solve return VFVM_ERR_TIMEOUT.  vfvm_check_bounded_wait runs that
barrier in a team told to expect one CTA more than was launched, so the wait
cannot complete and must expire; afterwards a solve and a CSR linear solve on
the same context still succeed.  Nothing traps, faults or hangs.
"""
import ctypes

import numpy as np
import pytest

from gpu_cases import lin

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ctas", [1, 4])
def test_expired_wait_returns_timeout_and_context_survives(vfvm, oracle, ctas):
    lib = vfvm._lib.load()
    st = ctypes.c_int32(-1)
    ms = ctypes.c_float(0.0)
    assert lib.vfvm_check_bounded_wait(ctas, ctypes.byref(st), ctypes.byref(ms)) == 0
    assert st.value == vfvm._lib.ERR_TIMEOUT
    assert 0.0 < ms.value < 60000.0
    # the context is still usable: a persistent-engine Newton solve agrees with the oracle
    g = vfvm.simplexgrid(lin(16), lin(16))
    sys = vfvm.System(g, vfvm.Physics("nlpoisson"))
    U = vfvm.solve(sys, inival=0.0, control=vfvm.SolverControl(engine="persistent"))
    uo, _ = oracle.solve_step(oracle.OracleSystem(g, "nlpoisson"), np.zeros(g.nnodes), oracle.Control())
    assert np.max(np.abs(U.ravel() - uo)) <= 1e-8 * np.max(np.abs(uo))


def test_bounded_wait_rejects_bad_input(vfvm):
    lib = vfvm._lib.load()
    st = ctypes.c_int32(0)
    assert lib.vfvm_check_bounded_wait(0, ctypes.byref(st), None) == vfvm._lib.ERR_INPUT
