"""Variable-step BDF with CVODE's error test and step-size / order rules
(params adaptive = 1; the role of CVODESolver, samrai/CVODESolver.cc:
112-258, driven one step at a time as QuatIntegrator.cc:1571-1596 drives
it) on the GPU against the same algorithm in the CPU oracle: the same
accepted steps (sizes within 1e-8 relative, the same orders, error-test
and Newton failures), FP64 fields within 1e-10 per field at the stop time;
the mixed path within 1e-5 of the oracle at the same stop time (its own
step sequence).  set_temperature: f(y) after a temperature change equals
f(y) of a stepper created at that temperature."""
import numpy as np
import pytest

import oracle as O
from ampe_gb300 import configs, initial
from ampe_gb300.stepper import ImplicitStepper

pytestmark = pytest.mark.gpu


def case(name):
    if name == "dilute2d":
        n = 64
        return configs.dilute2d(n), initial.dilute2d_state(n, seed=1, radius=12)
    n = 16
    return (configs.calphad3d(n, seed=3, T_run=1500.0),
            initial.calphad3d_state(n, seed=2, nseeds=2, radius=4.5))


def params(precision=0, h0=0.01):
    p = configs.step_params(dt=h0, precond=2, mg_levels=3, atol=1e-6, precision=precision)
    p.adaptive = 1
    return p


def one_step_run(s, t_stop, n):
    hs, qs = [], []
    st = None
    for _ in range(n):
        r = s.advance_to(t_stop, 1)
        rc, st = r if isinstance(r, tuple) else (0, r)
        assert rc == 0
        hs.append(st["h_last"])
        qs.append(st["q_last"])
        if st["t"] >= t_stop:
            break
    return np.array(hs), qs, st


@pytest.mark.parametrize("name", ["dilute2d", "calphad3d"])
def test_adaptive_parity(cuda, name):
    m, (phi, c) = case(name)
    t_stop = 0.6
    o = O.OracleStepper(m, params())
    o.set_state(phi, c)
    ho, qo, so = one_step_run(o, t_stop, 200)
    g = ImplicitStepper(m, params())
    g.set_state(phi, c)
    hg, qg, sg = one_step_run(g, t_stop, 200)
    print("%s: %d steps, h %.3g .. %.3g, orders %s, error-test failures %d"
          % (name, len(ho), ho.min(), ho.max(), sorted(set(qo)), so["err_test_fails"]))
    assert len(ho) == len(hg) and qo == qg
    assert np.max(np.abs(hg - ho) / ho) <= 1e-8
    assert abs(sg["t"] - t_stop) < 1e-12 and abs(so["t"] - t_stop) < 1e-12
    for k in ("newton_iters", "gmres_iters", "err_test_fails", "newton_fail"):
        assert sg[k] == so[k], (k, sg[k], so[k])
    assert max(qo) == 2 and ho.max() > 2 * ho.min()  # the controller did act
    for a, b in zip(g.get_state(), o.get_state()):
        assert O.rel_l2(a, b) <= 1e-10
    gm = ImplicitStepper(m, params(precision=1))
    gm.set_state(phi, c)
    one_step_run(gm, t_stop, 200)
    for a, b in zip(gm.get_state()[:2], o.get_state()[:2]):
        assert O.rel_l2(a, b) <= 1e-5


def test_set_temperature(cuda):
    m, (phi, c) = case("calphad3d")
    p = configs.step_params(dt=0.1, precond=2, mg_levels=3, atol=1e-6)
    g = ImplicitStepper(m, p)
    g.set_state(phi, c)
    g.set_temperature(1420.0, m.gradT)
    f1 = g.eval_rhs()
    m2 = configs.calphad3d(16, seed=3, T_run=1500.0)
    m2.T0 = 1420.0
    g2 = ImplicitStepper(m2, p)
    g2.set_state(phi, c)
    f2 = g2.eval_rhs()
    o = O.OracleStepper(m, p)
    o.set_state(phi, c)
    o.set_temperature(1420.0, m.gradT)
    fo = o.eval_rhs()
    for a, b, r in zip(f1, f2, fo):
        assert np.array_equal(a, b)
        assert O.rel_l2(a, r) <= 1e-11
