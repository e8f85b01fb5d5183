"""The reference's regression case tests/SingleGrainGrowthAuNi (test2d.py +
2d.input) as a model and an initial state for tests/kkscomposition.py's
run_adaptive.

An AuNi CALPHAD nucleus of radius 16 cells at the corner of a 64^2 box
(1.8 um, zero-slope boundaries), c = 0.096 inside and the balance of a
nominal 0.25 outside (utils/make_nuclei.py with "--nx 64 --ny 64 --nz 1
-r 16 --center0 0,0,0 -c 0.25 --concentration-in 0.096"), epsilon 0.25,
well scale 2.5, phase mobility 6.4, "pbg" energy and composition
interpolation, linear diffusion interpolation and arithmetic face
averages (QuatModelParameters.cc:886-1041 defaults), EBS composition flux
with the deck's default diffusion_type "composition_dependent": D_L, D_S
from the database's atomic mobilities at the face means of cL, cS
(QuatModelParameters.cc:238-249, MobilityCompositionDiffusionStrategy),
molar volume 7.68e-6, T = 1450 K - 200 K per unit time down to 1220 K,
atol 1e-5 (2d.input:24-92).  The reference expects the solid volume
fraction 0.32 +- 0.01 once t passes 0.3 (test2d.py:55-64; the mean of phi,
QuatModel::evaluateVolumeSolid) and the composition integral over the
3.24 um^2 box constant to 1e-4 (test2d.py:38-46).

The zero-slope 64^2 box is run as its mirror image, a 128^2 periodic
level (cell-centred zero-slope ghosts are the mirror images of the
interior cells).
"""
import json
import os

import numpy as np

from ampe_gb300 import abi, configs
from ampe_gb300.calphad_db import apply_database

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

LENGTH = 1.8
DRIFT_TOL = 1.0e-4 / LENGTH ** 2
SOLID_TARGET, SOLID_TOL = 0.32, 1.0e-2
ATOL = 1.0e-5
FIXTURE = os.path.join(GOLD, "singlegrain_oracle.json")
INTERVAL = 0.02  # the deck's ScalarDiagnostics interval (2d.input:68-71)


def initial_state(nh=64, radius=16.0, c_in=0.096, c_nominal=0.25):
    x = np.arange(nh) + 0.5
    X, Y = np.meshgrid(x, x, indexing="ij")
    ph = (np.sqrt(X ** 2 + Y ** 2) - radius < 0).astype(float)
    vs = ph.sum()
    vol = float(nh ** 2)
    c_out = (c_nominal * vol - c_in * vs) / (vol - vs)
    c = c_in * ph + c_out * (1.0 - ph)

    def mirror(a):
        for ax in range(2):
            a = np.concatenate([np.flip(a, ax), a], axis=ax)
        return np.ascontiguousarray(a.T).reshape(1, 2 * nh, 2 * nh)  # (z, y, x)

    return mirror(ph), mirror(c)


def model(nh=64):
    n = 2 * nh
    m = configs._blank_model(2, (n, n))
    with open(os.path.join(GOLD, "calphad_AuNi.json")) as f:
        apply_database(m, json.load(f))
    m.thermo = abi.THERMO_CALPHAD
    m.conc_diffusion = abi.DIFF_MOBILITY
    for d in range(2):
        m.dx[d] = LENGTH / nh
    m.epsilon_phi = 0.25
    m.phase_well_scale = 2.5
    m.phase_mobility = 6.4
    ivm = 1.0e-6 / 7.68e-6
    m.inv_molar_volume[0] = m.inv_molar_volume[1] = ivm
    m.energy_interp, m.conc_interp, m.diff_interp = b"p", b"p", b"l"
    m.avg_type, m.well_type = b"a", b"d"
    m.newton_max_its = 50
    m.temp_mode = abi.TEMP_CONSTANT
    m.T0 = 1450.0
    return m


def case(nh=64):
    return model(nh), initial_state(nh, radius=16.0 * nh / 64)


def block_means(a, b=8):
    """Means over b^2 blocks of a (1, y, x) level: a small summary of a
    field that a fixture can hold."""
    n1, n0 = a.shape[-2] // b, a.shape[-1] // b
    return a.reshape(n1, b, n0, b).mean(axis=(1, 3))


def run(make_stepper, precision=0, nh=64):
    """The deck's integration of the case (kkscomposition.run_adaptive:
    variable steps at atol 1e-5, rtol 1e-7, every f(t, y) at the deck's
    T(t)) to t = 0.3."""
    import kkscomposition as K

    return K.run_adaptive(make_stepper, atol=ATOL, precision=precision, case=case(nh),
                          interval=INTERVAL, mg_levels=4 if nh >= 32 else 3)
