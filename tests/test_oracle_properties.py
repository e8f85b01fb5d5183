"""Properties of the oracle stepper that hold independently of any golden
value (CPU): second-order convergence in the time step (BDF2 after the BDF1
start, CVODE's max order 2), conservation of the composition integral by
both composition flux forms, and unit quaternions after the normalisation
projection (QuatIntegrator.cc:3911-3940).  The GPU steppers reproduce the
oracle's steps to 1e-10, so the properties carry over to them."""
import numpy as np
import pytest

import oracle as O
from ampe_gb300 import abi, configs, initial


def test_second_order_in_time():
    m = configs.dilute2d(24)
    phi, c = initial.dilute2d_state(24, seed=1, radius=6)
    res = {}
    for dt in (0.04, 0.02, 0.01):
        p = configs.step_params(dt=dt, precond=2, mg_levels=2, atol=1e-10)
        p.max_newton = 6  # Newton error far below the truncation error
        o = O.OracleStepper(m, p)
        o.set_state(phi, c)
        rc, st = o.advance(int(round(0.4 / dt)))
        assert rc == 0 and st["step_retries"] == 0
        res[dt] = o.get_state()[:2]
    for f in range(2):
        e1 = np.linalg.norm(res[0.04][f] - res[0.02][f])
        e2 = np.linalg.norm(res[0.02][f] - res[0.01][f])
        assert 3.5 < e1 / e2 < 4.6, (f, e1 / e2)


@pytest.mark.parametrize("form", [abi.CONC_EBS, abi.CONC_KKS])
def test_composition_conserved(form):
    m = configs.calphad3d(12, seed=3, T_run=1500.0)
    m.conc_form = form
    phi, c = initial.calphad3d_state(12, seed=2, nseeds=2, radius=3.5)
    p = configs.step_params(dt=0.1, precond=2, mg_levels=2, atol=1e-8)
    o = O.OracleStepper(m, p)
    o.set_state(phi, c)
    rc, _ = o.advance(4)
    assert rc == 0
    assert abs(o.get_state()[1].mean() - c.mean()) < 1e-10


def test_quaternions_stay_unit():
    m = configs.polycrystal3d(12, seed=3, T=1500.0)
    phi, c, q = initial.polycrystal_state(12, ngrains=3, seed=1, channel=3.0)
    p = configs.step_params(dt=0.1, precond=2, mg_levels=2, atol=1e-6)
    o = O.OracleStepper(m, p)
    o.set_state(phi, c)
    o.set_quat(q)
    rc, _ = o.advance(3)
    assert rc == 0
    qn = o.get_quat()
    assert np.allclose(np.linalg.norm(qn, axis=0), 1.0, atol=1e-12)
    assert np.abs(qn - q).max() > 0.0  # the orientation field evolved
