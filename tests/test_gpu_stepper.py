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


def _mobility_case():
    """SingleGrainGrowthAuNi (tests/singlegrain.py) at a quarter of its
    resolution: the composition-dependent diffusivities of the atomic
    mobilities on the stepper's path."""
    import singlegrain as SG

    return SG.case(16)


def test_mobility_rhs_parity(cuda):
    m, (phi, c) = _mobility_case()
    p = configs.step_params(precond=2, mg_levels=3)
    o = O.OracleStepper(m, p)
    o.set_state(phi, c)
    g = ImplicitStepper(m, p)
    g.set_state(phi, c)
    fo, fg = o.eval_rhs(), g.eval_rhs()
    assert O.rel_l2(fg[0], fo[0]) <= 1e-11
    assert O.rel_l2(fg[1], fo[1]) <= 1e-11
    # the mobility diffusivities differ from the (unused) Arrhenius constants
    m2 = _mobility_case()[0]
    m2.conc_diffusion = 0
    a = O.OracleStepper(m2, p)
    a.set_state(phi, c)
    assert O.rel_l2(a.eval_rhs()[1], fo[1]) > 1e-3


@pytest.mark.parametrize("precond", [1, 2])
def test_mobility_steps_parity(cuda, precond):
    m, (phi, c) = _mobility_case()
    p = configs.step_params(dt=2e-4, precond=precond, mg_levels=3, atol=1e-5)
    o = O.OracleStepper(m, p)
    o.set_state(phi, c)
    rc, so = o.advance(4)
    assert rc == 0
    g = ImplicitStepper(m, p)
    g.set_state(phi, c)
    sg = g.advance(4)
    for k in ("steps", "newton_iters", "gmres_iters", "rhs_evals", "precond_solves", "fac_cycles"):
        assert sg[k] == so[k], (k, sg[k], so[k])
    for a, b in zip(g.get_state(), o.get_state()):
        assert O.rel_l2(a, b) <= 1e-10


def test_mobility_mixed_steps(cuda):
    """The mixed path (FP32 kernels, face weights from the FP32 cL, cS with
    the mobility diffusivities in FP64) against the FP64 oracle."""
    m, (phi, c) = _mobility_case()
    p = configs.step_params(dt=2e-4, precond=2, mg_levels=3, atol=1e-5)
    o = O.OracleStepper(m, p)
    o.set_state(phi, c)
    assert o.advance(4)[0] == 0
    p.precision = 1
    g = ImplicitStepper(m, p)
    g.set_state(phi, c)
    g.advance(4)
    xo = o.get_state()
    xg = g.get_state()
    for f in range(2):
        err = O.rel_l2(xg[f], xo[f])
        print("mobility mixed field %d rel L2 %.2e" % (f, err))
        assert err <= 2e-6


def test_mobility_refused_forms(cuda):
    from ampe_gb300._native import AmpeError

    m, _ = _mobility_case()
    p = configs.step_params(dt=2e-4)
    m.conc_form = 1  # "kks" form: its own diffusivities
    with pytest.raises(AmpeError):
        ImplicitStepper(m, p)
    m, _ = _mobility_case()
    m.mobility.q[0][0][0][1] = 0.0  # ln(0) of a mobility term
    with pytest.raises(AmpeError):
        ImplicitStepper(m, p)


def _ramp_case():
    """The reduced SingleGrainGrowthAuNi case with a steep temperature ramp
    that reaches its target within the test's steps: T0(t) = 1450 K -
    2e4 K t, held at 1440 K from t = 5e-4."""
    m, state = _mobility_case()
    m.T0, m.dTdt, m.T_target = 1450.0, -2.0e4, 1440.0
    return m, state


@pytest.mark.parametrize("adaptive", [False, True])
def test_temperature_ramp_parity(cuda, adaptive):
    """Every f(t, y) at the model's T0(t) (QuatIntegrator.cc:3191,
    ScalarTemperatureStrategy.cc:57-73), fixed and variable steps, against
    the oracle: same counts, fields within 1e-10."""
    m, (phi, c) = _ramp_case()
    p = configs.step_params(dt=2e-4, precond=2, mg_levels=3, atol=1e-5)
    p.adaptive = 1 if adaptive else 0
    o = O.OracleStepper(m, p)
    o.set_state(phi, c)
    g = ImplicitStepper(m, p)
    g.set_state(phi, c)
    if adaptive:
        rc, so = o.advance_to(8e-4, 100)
        assert rc == 0
        sg = g.advance_to(8e-4, 100)
        assert abs(sg["t"] - 8e-4) < 1e-15
    else:
        rc, so = o.advance(4)
        assert rc == 0
        sg = g.advance(4)
    for k in ("steps", "newton_iters", "gmres_iters", "rhs_evals", "fac_cycles"):
        assert sg[k] == so[k], (k, sg[k], so[k])
    xo, xg = o.get_state(), g.get_state()
    for a, b in zip(xg, xo):
        assert O.rel_l2(a, b) <= 1e-10
    # the ramp changes the result: the same steps at a fixed 1450 K
    m2, _ = _mobility_case()
    f = ImplicitStepper(m2, p)
    f.set_state(phi, c)
    if adaptive:
        f.advance_to(8e-4, 100)
    else:
        f.advance(4)
    assert O.rel_l2(f.get_state()[0], xg[0]) > 1e-6
    # the ramp owns the temperature
    from ampe_gb300._native import AmpeError

    with pytest.raises(AmpeError):
        g.set_temperature(1400.0)
