"""The ODE/DAE form of a system (src/vfvm_diffeq_interface.jl:10-112) on the
GPU against the oracle: eval_rhs = -F and eval_jacobian = -J at tstep = Inf,
and the mass matrix (storage Jacobian at U = 0), within 1e-12 row-relative;
for a linear storage the implicit Euler residual equals -rhs + M (u - uold)/dt."""
import math

import numpy as np
import pytest

from gpu_cases import case, random_state

pytestmark = pytest.mark.gpu
TOL = 1e-12


def pair(vfvm, oracle, name):
    c = case(vfvm, name)
    sys = vfvm.System(c["grid"], vfvm.Physics(c["kind"], c["params"], c["nodedata"]))
    bf = bv = None
    if c["legacy"] is not None:
        bf, bv = c["legacy"]
        for i in range(bf.shape[0]):
            for r in range(bf.shape[1]):
                if bf[i, r] == 1e30:
                    vfvm.boundary_dirichlet(sys, i + 1, r + 1, bv[i, r])
    osys = oracle.OracleSystem(c["grid"], c["kind"], c["params"], nodedata=c["nodedata"], bfactors=bf, bvalues=bv)
    return c, sys, osys


@pytest.mark.parametrize("name", ["porous", "ex161", "surface_heat2d", "surface_heat3d", "ex110"])
def test_mass_matrix_vs_oracle(vfvm, oracle, name):
    c, sys, osys = pair(vfvm, oracle, name)
    M = vfvm.mass_matrix(sys).toarray()
    Mo = osys.mass_matrix().toarray()
    scale = np.maximum(np.max(np.abs(Mo), axis=1, keepdims=True), 1e-300)
    assert np.all(np.abs(M - Mo) <= TOL * scale)
    assert np.max(np.abs(Mo)) > 0


@pytest.mark.parametrize("name", ["porous", "ex161", "kappa_exp", "bipolar"])
def test_rhs_and_jacobian_vs_oracle(vfvm, oracle, name):
    c, sys, osys = pair(vfvm, oracle, name)
    U = random_state(c, sys.nspec, np.random.default_rng(8))
    rhs = vfvm.eval_rhs(sys, U, t=c["t"]).ravel(order="F")
    Jr = vfvm.eval_jacobian(sys, U, t=c["t"]).toarray()
    Fo, Jo = osys.assemble(U.ravel(order="F"), None, c["t"], math.inf, 0.0)
    Jo = Jo.toarray()
    rowscale = np.maximum(np.abs(Fo), np.abs(Jo) @ np.abs(U.ravel(order="F")))
    assert np.all(np.abs(rhs + Fo) <= TOL * rowscale + 1e-300)
    jscale = np.maximum(np.max(np.abs(Jo), axis=1, keepdims=True), 1e-300)
    assert np.all(np.abs(Jr + Jo) <= TOL * jscale)


def test_implicit_euler_from_the_ode_form(vfvm, oracle):
    """porous medium (storage u): F(u, uold, dt) = -rhs(u) + M (u - uold) / dt."""
    c, sys, _ = pair(vfvm, oracle, "porous")
    rng = np.random.default_rng(3)
    U = random_state(c, 1, rng)
    Uold = random_state(c, 1, rng)
    dt = 1e-3
    F, _ = vfvm.evaluate_residual_and_jacobian(sys, U, tstep=dt, uold=Uold)
    M = vfvm.mass_matrix(sys)
    G = -vfvm.eval_rhs(sys, U).ravel(order="F") + M @ (U - Uold).ravel(order="F") / dt
    assert np.allclose(F.ravel(order="F"), G, rtol=1e-12, atol=1e-12 * np.max(np.abs(G)))
