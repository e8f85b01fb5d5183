"""GPU implicit stepper against the CPU oracle stepper: same seeded inputs,
same algorithm (BDF, Newton, GMRES, FAC/multigrid), FP64.  Parity bar:
relative L2 <= 1e-10 per field with identical Newton / GMRES counts."""
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
    m = configs.calphad3d(n, seed=3, T_run=1500.0)
    return m, initial.calphad3d_state(n, seed=2, nseeds=2, radius=4.5)


@pytest.mark.parametrize("name", ["dilute2d", "calphad3d"])
def test_eval_rhs_parity(cuda, name):
    m, (phi, c) = case(name)
    p = configs.step_params(precond=2, mg_levels=3)
    o = O.OracleStepper(m, p)
    o.set_state(phi, c)
    g = ImplicitStepper(m, p)
    g.set_state(phi, c)
    fo = o.eval_rhs()
    fg = g.eval_rhs()
    assert O.rel_l2(fg[0], fo[0]) <= 1e-11
    assert O.rel_l2(fg[1], fo[1]) <= 1e-11


@pytest.mark.parametrize("name", ["dilute2d", "calphad3d"])
@pytest.mark.parametrize("precond", [0, 1, 2])
def test_steps_parity(cuda, name, precond):
    m, (phi, c) = case(name)
    p = configs.step_params(dt=0.1, precond=precond, mg_levels=3)
    nsteps = 4
    o = O.OracleStepper(m, p)
    o.set_state(phi, c)
    rc, so = o.advance(nsteps)
    assert rc == 0
    g = ImplicitStepper(m, p)
    g.set_state(phi, c)
    sg = g.advance(nsteps)
    for k in ("steps", "newton_iters", "gmres_iters", "rhs_evals", "precond_solves", "fac_cycles"):
        assert sg[k] == so[k], (k, sg[k], so[k])
    xo = o.get_state()
    xg = g.get_state()
    for a, b in zip(xg, xo):
        assert O.rel_l2(a, b) <= 1e-10


def test_deterministic_and_conservative(cuda):
    m, (phi, c) = case("dilute2d")
    p = configs.step_params(dt=0.1, precond=1)
    out = []
    for _ in range(2):
        g = ImplicitStepper(m, p)
        g.set_state(phi, c)
        g.advance(6)
        out.append(g.get_state())
        g.close()
    for a, b in zip(*out):
        assert np.array_equal(a, b)
    assert abs(out[0][1].mean() - c.mean()) < 1e-9
    assert out[0][0].max() <= 1.05 and out[0][0].min() >= -0.05
