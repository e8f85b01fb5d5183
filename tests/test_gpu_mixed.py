"""Mixed-precision path (FP32 KKS Newton / RHS / analytic Jacobian / FP32
multigrid inside the FP64 Newton-Krylov iteration) against the FP64 oracle.

Tolerances: the analytic FP32 Jacobian-vector product within 1e-5 relative
L2 of the oracle's FP64 analytic product; the FP64 path's finite-difference
product within 1e-9 of the oracle's; whole steps of the mixed path within
2e-6 relative L2 per field of the oracle's FP64 steps at atol 1e-6."""
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


@pytest.mark.parametrize("name", ["dilute2d", "calphad3d"])
def test_jv_products(cuda, name):
    m, (phi, c) = case(name)
    rng = np.random.default_rng(11)
    v = rng.standard_normal(2 * m.cells()) * 1e-3
    p64 = configs.step_params(precond=2, mg_levels=3, atol=1e-6)
    o = O.OracleStepper(m, p64)
    o.set_state(phi, c)
    o.advance(2)
    ph, cc, cl, cs = o.get_state()
    g64 = ImplicitStepper(m, p64)
    g64.set_state(ph, cc, cl, cs)
    o.set_state(ph, cc, cl, cs)
    assert O.rel_l2(g64.jv(v, 0.1), o.jv(v, 0.1, 0)) <= 1e-9
    pm = configs.step_params(precond=2, mg_levels=3, atol=1e-6, precision=1)
    gm = ImplicitStepper(m, pm)
    gm.set_state(ph, cc, cl, cs)
    an = o.jv(v, 0.1, 1)
    out = gm.jv(v, 0.1)
    assert O.rel_l2(out - v, an - v) <= 1e-5


@pytest.mark.parametrize("name", ["dilute2d", "calphad3d"])
def test_mixed_steps_vs_oracle(cuda, name):
    m, (phi, c) = case(name)
    nsteps = 6
    p64 = configs.step_params(dt=0.1, precond=2, mg_levels=3, atol=1e-6)
    o = O.OracleStepper(m, p64)
    o.set_state(phi, c)
    rc, so = o.advance(nsteps)
    assert rc == 0
    pm = configs.step_params(dt=0.1, precond=2, mg_levels=3, atol=1e-6, precision=1)
    g = ImplicitStepper(m, pm)
    g.set_state(phi, c)
    sg = g.advance(nsteps)
    assert sg["steps"] == nsteps and sg["kks_fail"] == 0
    xo, xg = o.get_state(), g.get_state()
    errs = [O.rel_l2(a, b) for a, b in zip(xg[:2], xo[:2])]
    print(name, "mixed vs FP64 oracle rel L2 (phi, c):", errs, sg)
    assert max(errs) <= 2e-6


def test_mixed_fp64_cells_near_bounds(cuda):
    # compositions within 1e-3 of 0 switch the KKS solve to FP64
    m = configs.dilute2d(32)
    phi, c = initial.dilute2d_state(32, seed=3, radius=8, c0=5e-4, noise=1e-4)
    pm = configs.step_params(dt=0.05, precond=2, mg_levels=3, atol=1e-6, precision=1)
    g = ImplicitStepper(m, pm)
    g.set_state(phi, c)
    sg = g.advance(2)
    assert sg["kks_fp64_cells"] > 0 and sg["kks_fail"] == 0
    p64 = configs.step_params(dt=0.05, precond=2, mg_levels=3, atol=1e-6)
    o = O.OracleStepper(m, p64)
    o.set_state(phi, c)
    o.advance(2)
    for a, b in zip(g.get_state()[:2], o.get_state()[:2]):
        assert O.rel_l2(a, b) <= 2e-6
