"""The oracle's Kim phase mobility (KimMobilityStrategyInfMob.cc:49-80,
kks_mobility_factor in KKStools.cc:13-30) against a numpy restatement:
M = 16 w / (3 eps^2 a2) / ((cL - cS)^2 f_L''(cL) / (D0 exp(-Q0/RT)) x
1e-6/Vm), f_L'' from the oracle's own second derivative (pinned against
finite differences of the free energy in test_oracle_kats).  Bar 1e-13."""
import ctypes as C

import numpy as np

import oracle as O
from ampe_gb300 import configs

R = 8.314472


def test_kim_mobility(orc):
    m = configs.calphad3d(6, seed=3, T_run=1500.0)
    rng = np.random.default_rng(8)
    shp = m.interior_shape()
    cl = O.ghosted(m, rng.uniform(0.3, 0.5, shp))
    cs = O.ghosted(m, rng.uniform(0.1, 0.25, shp))
    factor = 16 * m.phase_well_scale / (3 * m.epsilon_phi ** 2 * (47.0 / 60.0))
    mob = np.zeros_like(cl)
    D0, Q0, mv = 2.5, 4.0e4, 7.68e-6
    orc.orc_kim_mobility(C.byref(m), None, O.ptr(cl), O.ptr(cs), factor, D0, Q0, mv,
                         O.ptr(mob))
    g = m.ng
    x = np.arange(-g, m.n[0] + g)
    T = m.T0 + m.gradT * ((x % m.n[0]) + 0.5) * m.dx[0]
    T = np.broadcast_to(T, cl.shape)
    d2 = np.vectorize(lambda c, t: orc.orc_d2fdc2(C.byref(m), t, c, 0))(cl, T)
    zeta = (cl - cs) * d2 * (cl - cs) / (D0 * np.exp(-Q0 / (R * T))) * (1e-6 / mv)
    assert O.rel_l2(mob, factor / zeta) <= 1e-13
