"""The oracle's variable-step BDF (params adaptive = 1, CVODE's error test
and step-size / order rules) on CPU: it lands on the stop time exactly in
one-step calls, raises the order to 2 and grows the step on a smooth
solution, and its error against a tight-tolerance run shrinks with the
tolerance; the fixed-step mode is untouched by the new fields."""
import numpy as np

import oracle as O
from ampe_gb300 import configs, initial

N = 24


def _case():
    return configs.dilute2d(N), initial.dilute2d_state(N, seed=1, radius=6)


def _run(atol, t_stop=0.4, h0=0.01):
    m, (phi, c) = _case()
    p = configs.step_params(dt=h0, precond=2, mg_levels=2, atol=atol)
    p.adaptive = 1
    o = O.OracleStepper(m, p)
    o.set_state(phi, c)
    hs, qs = [], []
    for _ in range(400):
        rc, st = o.advance_to(t_stop, 1)
        assert rc == 0
        hs.append(st["h_last"])
        qs.append(st["q_last"])
        if st["t"] >= t_stop:
            break
    assert abs(st["t"] - t_stop) < 1e-12
    return o.get_state()[:2], np.array(hs), qs, st


def test_adaptive_error_control():
    ref, _, _, _ = _run(1e-9)
    errs = []
    for atol in (1e-5, 1e-7):
        x, hs, qs, st = _run(atol)
        errs.append(max(O.rel_l2(a, b) for a, b in zip(x, ref)))
        if atol == 1e-5:
            assert max(qs) == 2 and hs.max() > 2 * hs.min()
    assert errs[1] < errs[0] / 5, errs


def test_fixed_mode_unchanged():
    m, (phi, c) = _case()
    p = configs.step_params(dt=0.05, precond=2, mg_levels=2, atol=1e-6)
    assert p.adaptive == 0
    o = O.OracleStepper(m, p)
    o.set_state(phi, c)
    rc, st = o.advance(3)
    assert rc == 0 and abs(st["t"] - 0.15) < 1e-12
    assert st["h_last"] == 0.05 and st["q_last"] == 2
