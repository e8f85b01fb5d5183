"""The reference's regression case tests/KKScomposition (test3d.py +
3d.input) as a model, an initial state and a time-stepping loop that any
stepper with set_state / advance / get_state / close can run (the CPU
oracle or the CUDA library).

An AuNi CALPHAD nucleus of radius 16 cells at the corner of a 32^3 box
(0.9 um, zero-slope boundaries), c = 0.096 inside and the balance of a
nominal 0.25 outside (utils/make_nuclei.py with "-r 16 --center0 0,0,0
-c 0.25 --concentration-in 0.096"), sigma 0.372678, delta 0.035 (eps =
sqrt(6 sigma delta), well scale 3 sigma / (16 delta),
QuatModelParameters.cc:842-845), mobility 6.4, D_L 1224.23, D_S 0.125, EBS
composition flux with linear diffusion interpolation, molar volume 7.68e-6
(energies x 1e-6 / Vm), T = 1450 K - 200 K per unit time.  The reference
expects the solid volume fraction 0.33 +- 0.01 at t = 0.3 (test3d.py:55-62;
mean of phi, QuatModel::evaluateVolumeSolid) and the composition integral
over the 0.729 um^3 box constant to 1e-4 (test3d.py:38-46).

The deck sets no diffusion_type, so the reference derives composition-
dependent diffusivities from the database's atomic mobilities
(MobilityCompositionDiffusionStrategy, QuatModelParameters.cc:238-246);
this run uses the deck's D_L and D_S, which the deck's comment gives as
that model's values at 1450 K (3d.input:51-53).

The zero-slope 32^3 box is run as its mirror image, a 64^3 periodic level
(cell-centred zero-slope ghosts are the mirror images of the interior
cells).  Fixed-step BDF1 with a geometric start-up (the sharp initial
interface) and T updated per step.
"""
import json
import os

import numpy as np

from ampe_gb300 import abi, configs
from ampe_gb300.calphad_db import apply_database

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIXTURE = os.path.join(GOLD, "kkscomposition_oracle.json")
FIXTURE_MOBILITY = os.path.join(GOLD, "kkscomposition_mobility_oracle.json")

# composition integral tolerance of test3d.py:44-46 (1e-4 on the integral
# over the 0.9^3 um^3 box) as a tolerance on the mean composition
DRIFT_TOL = 1.0e-4 / 0.9 ** 3
SOLID_TARGET, SOLID_TOL = 0.33, 1.0e-2


def initial_state(nh=32, radius=16.0, c_in=0.096, c_nominal=0.25):
    x = np.arange(nh) + 0.5
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    ph = (np.sqrt(X ** 2 + Y ** 2 + Z ** 2) - radius < 0).astype(float)
    vs = ph.sum()
    vol = float(nh ** 3)
    c_out = (c_nominal * vol - c_in * vs) / (vol - vs)
    c = c_in * ph + c_out * (1.0 - ph)

    def mirror(a):
        for ax in range(3):
            a = np.concatenate([np.flip(a, ax), a], axis=ax)
        return np.ascontiguousarray(a.transpose(2, 1, 0))  # (z, y, x)

    return mirror(ph), mirror(c)


def model(nh=32, mobility=False):
    """The deck's model with its D_L, D_S constants, or (mobility=True) with
    the reference's actual diffusivities for it: "composition_dependent",
    from the database's atomic mobilities, the default for "ebs" when the
    deck names no diffusion_type (its D_L, D_S are then not read,
    QuatModelParameters.cc:238-260)."""
    n = 2 * nh
    m = configs._blank_model(3, (n, n, n))
    with open(os.path.join(GOLD, "calphad_AuNi.json")) as f:
        apply_database(m, json.load(f))
    m.thermo = abi.THERMO_CALPHAD
    for d in range(3):
        m.dx[d] = 0.9 / nh
    sigma, delta = 0.372678, 0.035
    m.epsilon_phi = np.sqrt(6.0 * sigma * delta)
    m.phase_well_scale = 3.0 * sigma / delta / 16.0
    m.phase_mobility = 6.4
    m.D_liquid, m.D_solid = 1224.23, 0.125
    m.Q_liquid = m.Q_solid = 0.0
    ivm = 1.0e-6 / 7.68e-6
    m.inv_molar_volume[0] = m.inv_molar_volume[1] = ivm
    m.energy_interp, m.conc_interp, m.diff_interp = b"p", b"p", b"l"
    m.avg_type, m.well_type = b"a", b"d"
    m.newton_max_its = 50
    m.temp_mode = abi.TEMP_CONSTANT
    if mobility:
        m.conc_diffusion = abi.DIFF_MOBILITY
    return m


def block_means(a, b=4):
    """Means over b^3 blocks of a (z, y, x) cube: a small summary of a field
    that a fixture can hold."""
    n = a.shape[0] // b
    return a.reshape(n, b, n, b, n, b).mean(axis=(1, 3, 5))


def run(make_stepper, t_end=0.3, dt_max=2.0e-3, atol=1.0e-6, precision=0,
        interval=0.03, t_stop=None, mobility=False):
    """Advance the case to t_end with make_stepper(model, params) steppers.

    Returns a dict: per output time (every `interval`, as the deck's
    ScalarDiagnostics) the time, temperature, solid fraction and mean
    composition; the final phi and c; the number of accepted and rejected
    steps.  t_stop < t_end ends the run early (same step sequence);
    mobility selects model(mobility=True)."""
    m = model(mobility=mobility)
    phi, c = initial_state()
    cl = cs = None
    p = configs.step_params(dt=dt_max, precond=2, mg_levels=4, atol=atol,
                            precision=precision)
    p.max_order = 1
    t, k, dt_target, ramp = 0.0, 0, dt_max, True
    c0 = float(c.mean())
    out = {"t": [0.0], "T": [1450.0], "solid": [float(phi.mean())], "cmean": [c0],
           "steps": 0, "rejected": 0}
    next_out = interval
    t_last = t_end if t_stop is None else t_stop
    while t < t_last - 1e-12:
        dt = min(dt_target, t_end - t)
        if ramp:
            dt = min(dt, 1.0e-6 * 2.0 ** k)
            k += 1
        p.dt = dt
        m.T0 = 1450.0 - 200.0 * (t + dt)
        s = make_stepper(m, p)
        s.set_state(phi, c, cl, cs)
        st = s.advance(1)
        rc = st[0] if isinstance(st, tuple) else 0
        if rc != 0:
            s.close()
            dt_target, ramp = dt / 4.0, False
            out["rejected"] += 1
            continue
        phi, c, cl, cs = s.get_state()
        s.close()
        t += dt
        out["steps"] += 1
        if not ramp:
            dt_target = min(dt_max, dt_target * 1.25)
        if t >= next_out - 1e-9:
            out["t"].append(t)
            out["T"].append(m.T0)
            out["solid"].append(float(phi.mean()))
            out["cmean"].append(float(c.mean()))
            next_out += interval
    out["phi"], out["c"] = phi, c
    out["drift"] = float(c.mean()) - c0
    return out


T_START, DTDT, T_TARGET = 1450.0, -200.0, 1220.0  # 3d.input:20-25, 2d.input:24-29


def temperature(t):
    """ScalarTemperatureStrategy::getCurrentTemperature
    (ScalarTemperatureStrategy.cc:57-73) with the deck's 1450 K, -200 K per
    unit time and target 1220 K."""
    return max(T_START + DTDT * t, T_TARGET)


def run_adaptive(make_stepper, t_end=0.3, atol=1.0e-4, h0=1.0e-6, precision=0,
                 interval=0.03, max_steps=100000, case=None, mg_levels=4, ramp=True):
    """The deck's own integration: CVODE-style variable steps (orders 1-2,
    atol 1e-4 and rtol = atol / 100 as QuatIntegrator.cc:283-289 derives
    them from 3d.input:80-81, initial step h0), one accepted step per call
    (CV_ONE_STEP, QuatIntegrator.cc:1575) up to t_end, the temperature
    following the deck's scalar history inside the stepper (model fields
    T0, dTdt, T_target: every f(t, y) at temperature(t), as
    QuatIntegrator.cc:3191 sets it); ramp=False instead sets T from the
    host before each step, at the step's start time, and holds it within
    the step.  case = (model, (phi, c)) runs another case the same way.
    Returns the same record as run()."""
    if case is None:
        m = model()
        phi, c = initial_state()
    else:
        m, (phi, c) = case
    m.T0, m.dTdt, m.T_target = T_START, (DTDT if ramp else 0.0), T_TARGET
    p = configs.step_params(dt=h0, precond=2, mg_levels=mg_levels, atol=atol,
                            precision=precision)
    p.adaptive = 1
    s = make_stepper(m, p)
    s.set_state(phi, c)
    c0 = float(c.mean())
    out = {"t": [0.0], "T": [1450.0], "solid": [float(phi.mean())], "cmean": [c0],
           "steps": 0, "rejected": 0, "h": []}
    next_out, t = interval, 0.0
    st = None
    while t < t_end - 1e-12 and out["steps"] < max_steps:
        if not ramp:
            s.set_temperature(temperature(t))
        r = s.advance_to(t_end, 1)
        rc, st = r if isinstance(r, tuple) else (0, r)
        if rc != 0:
            raise RuntimeError("adaptive step failed at t = %g" % t)
        t = st["t"]
        out["steps"] += 1
        out["h"].append(st["h_last"])
        if t >= next_out - 1e-9 or t >= t_end - 1e-12:
            ph, cc = s.get_state()[:2]
            out["t"].append(t)
            out["T"].append(temperature(t))
            out["solid"].append(float(ph.mean()))
            out["cmean"].append(float(cc.mean()))
            while next_out <= t + 1e-9:
                next_out += interval
    phi, c = s.get_state()[:2]
    out["phi"], out["c"] = phi, c
    out["drift"] = float(c.mean()) - c0
    out["rejected"] = st["err_test_fails"] + st["newton_fail"] if st else 0
    out["newton_iters"] = st["newton_iters"] if st else 0
    s.close()
    return out
