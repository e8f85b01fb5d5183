"""Temperature in time and the adaptive stop time in the oracle stepper, on
the CPU.

* With the model's ramp (T0, dTdt, T_target) every f(t, y) is evaluated at
  T0(t) (QuatIntegrator::setTemperatureField, QuatIntegrator.cc:3191;
  ScalarTemperatureStrategy::getCurrentTemperature,
  ScalarTemperatureStrategy.cc:57-73).  A BDF1 step's Newton iterations
  then see T(t_{n+1}): four steps with the ramp equal four single steps of
  fresh steppers held at the end time's temperature, for a cooling ramp
  and a heating ramp that both reach their target inside the run.
* advance_to ends at its stop time: a second call with the same stop time
  takes no step, and a stop time before the current time sets none."""
import numpy as np
import pytest

import oracle as O
import singlegrain as SG
from ampe_gb300 import configs

DT = 2e-4


def _ramp(T0, dTdt, target, t):
    T = T0 + dTdt * t
    if dTdt < 0 and T < target:
        return target
    if target > 0 and dTdt > 0 and T > target:
        return target
    return T


@pytest.mark.parametrize("dTdt,target", [(-2.0e4, 1440.0), (2.0e4, 1460.0)])
def test_ramp_is_the_end_time_temperature(dTdt, target):
    m, (phi, c) = SG.case(16)
    m.T0, m.dTdt, m.T_target = 1450.0, dTdt, target
    p = configs.step_params(dt=DT, precond=2, mg_levels=3, atol=1e-5)
    p.max_order = 1
    o = O.OracleStepper(m, p)
    o.set_state(phi, c)
    rc, st = o.advance(4)
    assert rc == 0 and st["steps"] == 4
    ramped = o.get_state()
    ph, cc, cl, cs = phi, c, None, None
    for n in range(4):
        mf, _ = SG.case(16)
        mf.T0 = _ramp(1450.0, dTdt, target, (n + 1) * DT)
        s = O.OracleStepper(mf, p)
        s.set_state(ph, cc, cl, cs)
        assert s.advance(1)[0] == 0
        ph, cc, cl, cs = s.get_state()
    for a, b in zip(ramped, (ph, cc, cl, cs)):
        assert O.rel_l2(a, b) <= 1e-13
    # the target is reached inside the run: the ramp is not the fixed start
    mf, _ = SG.case(16)
    f = O.OracleStepper(mf, p)
    f.set_state(phi, c)
    f.advance(4)
    assert O.rel_l2(f.get_state()[0], ramped[0]) > 1e-6


def test_stop_time():
    m, (phi, c) = SG.case(16)
    p = configs.step_params(dt=DT, precond=2, mg_levels=3, atol=1e-5)
    p.adaptive = 1
    o = O.OracleStepper(m, p)
    o.set_state(phi, c)
    rc, st = o.advance_to(8e-4, 1000)
    assert rc == 0 and st["t"] == pytest.approx(8e-4, rel=1e-12, abs=0)
    n = st["steps"]
    assert n < 1000
    rc, st = o.advance_to(8e-4, 1000)  # reached: no step
    assert rc == 0 and st["steps"] == n
    rc, st = o.advance_to(1e-4, 3)  # in the past: no stop time, 3 steps
    assert rc == 0 and st["steps"] == n + 3 and st["t"] > 8e-4
