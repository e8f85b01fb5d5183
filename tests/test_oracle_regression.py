"""End-to-end pin of the oracle stepper on the reference's own regression
case tests/KKScomposition (test3d.py + 3d.input): an AuNi CALPHAD nucleus of
radius 16 cells at the corner of a 32^3 box (0.9 um, zero-slope boundaries),
c = 0.096 inside and the balance of a nominal 0.25 outside
(utils/make_nuclei.py with "-r 16 --center0 0,0,0 -c 0.25
--concentration-in 0.096"), sigma 0.372678, delta 0.035 (eps = sqrt(6 sigma
delta), well scale 3 sigma / (16 delta), QuatModelParameters.cc:842-845),
mobility 6.4, D_L 1224.23, D_S 0.125, EBS composition flux with linear
diffusion interpolation, molar volume 7.68e-6 (energies x 1e-6 / Vm), T =
1450 K - 200 K per unit time.  The reference expects the solid volume
fraction 0.33 +- 0.01 at t = 0.3 (test3d.py:55-62; mean of phi,
QuatModel::evaluateVolumeSolid).

The deck sets no diffusion_type, so the reference derives composition-
dependent diffusivities from the database's atomic mobilities
(MobilityCompositionDiffusionStrategy, QuatModelParameters.cc:238-246);
this run uses the deck's D_L and D_S, which the deck's comment gives as
that model's values at 1450 K (3d.input:51-53).

The zero-slope 32^3 box is run as its mirror image, a 64^3 periodic level
(cell-centred zero-slope ghosts are the mirror images of the interior
cells).  Fixed-step BDF1 with a geometric start-up (the sharp initial
interface) and T updated per step.  Measured: solid fraction 0.3343 at
t = 0.3, mean composition drift -4.3e-6 (79 minutes on 8 cores): opt-in
with AMPE_SLOW_TESTS=1."""
import json
import os

import numpy as np
import pytest

from ampe_gb300 import abi, configs
from ampe_gb300.calphad_db import apply_database

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

pytestmark = pytest.mark.skipif(os.environ.get("AMPE_SLOW_TESTS") != "1",
                                reason="long CPU run; set AMPE_SLOW_TESTS=1")


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


def model(nh=32):
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
    return m


def run(t_end=0.3, dt_max=2.0e-3, atol=1.0e-6):
    import oracle as O

    m = model()
    phi, c = initial_state()
    cl = cs = None
    p = configs.step_params(dt=dt_max, precond=2, mg_levels=4, atol=atol)
    p.max_order = 1
    t, k, dt_target, ramp = 0.0, 0, dt_max, True
    c0 = c.mean()
    while t < t_end - 1e-12:
        dt = min(dt_target, t_end - t)
        if ramp:
            dt = min(dt, 1.0e-6 * 2.0 ** k)
            k += 1
        p.dt = dt
        m.T0 = 1450.0 - 200.0 * (t + dt)
        s = O.OracleStepper(m, p)
        s.set_state(phi, c, cl, cs)
        rc, _ = s.advance(1)
        if rc != 0:
            s.close()
            dt_target, ramp = dt / 4.0, False
            continue
        phi, c, cl, cs = s.get_state()
        s.close()
        t += dt
        if not ramp:
            dt_target = min(dt_max, dt_target * 1.25)
    return float(phi.mean()), float(c.mean() - c0)


def test_kkscomposition_solid_fraction():
    solid, drift = run()
    print("solid fraction at t = 0.3: %.4f, mean composition drift %.2e" % (solid, drift))
    assert abs(drift) < 1.4e-4  # test3d.py:44-46: integral over 0.729 um^3 within 1e-4
    assert abs(solid - 0.33) <= 1.0e-2
