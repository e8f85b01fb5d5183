"""Failure handling of the implicit stepper, made on the host: no GPU fault,
trap or hang is involved.  A KKS solve capped at one Newton iteration
(reference: PhaseConcentrationsStrategy::computePhaseConcentrations returns
a negative count and its caller aborts, PhaseConcentrationsStrategy.cc:118)
is reported as a count of failed cells while the step goes on, as the
oracle does; a time step far beyond what one Newton iteration can take
(CVODE's convergence failure) ends in AMPE_ERR_NOT_CONVERGED after the
retries, with the state left at the last accepted step; afterwards the
same process and CUDA context run a normal step."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from ampe_gb300 import abi, configs, initial
from ampe_gb300.stepper import ImplicitStepper

pytestmark = pytest.mark.gpu


def small_case():
    m = configs.dilute2d(32)
    phi, c = initial.dilute2d_state(32, seed=1, radius=8)
    return m, phi, c


def test_kks_failures_counted(cuda):
    m, phi, c = small_case()
    m.newton_max_its = 1
    p = configs.step_params(dt=0.1, precond=2, mg_levels=2, atol=1e-6)
    o = O.OracleStepper(m, p)
    o.set_state(phi, c)
    rc_o, so = o.advance(2)
    g = ImplicitStepper(m, p)
    g.set_state(phi, c)
    st = abi.StepStats()
    rc = cuda.lib.ampe_stepper_advance(g._h, 2, C.byref(st))
    sg = st.as_dict()
    assert rc == 0 and rc_o == 0
    assert sg["steps"] == so["steps"] == 2
    assert sg["kks_fail"] > 0 and so["kks_fail"] > 0
    for a, b in zip(g.get_state(), o.get_state()):
        assert np.all(np.isfinite(a))
        assert O.rel_l2(a, b) <= 1e-8


def test_newton_failure_status(cuda):
    m, phi, c = small_case()
    p = configs.step_params(dt=200.0, precond=2, mg_levels=2, atol=1e-6)
    p.max_newton = 1
    o = O.OracleStepper(m, p)
    o.set_state(phi, c)
    rc_o, so = o.advance(2)
    assert rc_o != 0 and so["steps"] == 0
    g = ImplicitStepper(m, p)
    g.set_state(phi, c)
    st = abi.StepStats()
    rc = cuda.lib.ampe_stepper_advance(g._h, 2, C.byref(st))
    sg = st.as_dict()
    assert rc == abi.AMPE_ERR_NOT_CONVERGED
    assert sg["steps"] == 0 and sg["newton_fail"] > 0 and sg["step_retries"] > 0
    # the state is the last accepted one: the initial state
    ph, cc = g.get_state()[:2]
    assert np.array_equal(ph.ravel(), phi.ravel()) and np.array_equal(cc.ravel(), c.ravel())
    # the context is still usable: a normal step in the same process
    p2 = configs.step_params(dt=0.1, precond=2, mg_levels=2, atol=1e-6)
    g2 = ImplicitStepper(m, p2)
    g2.set_state(phi, c)
    assert g2.advance(1)["steps"] == 1
