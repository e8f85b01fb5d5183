"""The oracle's analytic Jacobian-vector product (the reference the mixed
GPU path's FP32 product is checked against) against the oracle's own
finite-difference product, formed as CVODE forms it (sigma = 1 / ||v||_WRMS,
QuatIntegrator.cc:3189-3267 holds the composition diffusivities and, in the
"kks" form, the coupling coefficient lagged in both), on CPU.  Bar: 1e-5
relative L2 per block of rows; the difference is the FD truncation error."""
import numpy as np
import pytest

import oracle as O
from ampe_gb300 import abi, configs, initial


def case(name):
    if name == "dilute2d":
        m = configs.dilute2d(32)
        phi, c = initial.dilute2d_state(32, seed=1, radius=8)
    else:
        m = configs.calphad3d(12, seed=3, T_run=1500.0)
        phi, c = initial.calphad3d_state(12, seed=2, nseeds=2, radius=3.5)
        if name == "calphad3d_kks":
            m.conc_form = abi.CONC_KKS
    return m, phi, c


@pytest.mark.parametrize("name", ["dilute2d", "calphad3d", "calphad3d_kks"])
def test_analytic_jv_matches_fd(orc, name):
    m, phi, c = case(name)
    p = configs.step_params(dt=0.1, precond=2, mg_levels=2, atol=1e-6)
    o = O.OracleStepper(m, p)
    o.set_state(phi, c)
    rc, _ = o.advance(2)
    assert rc == 0
    ph, cc, cl, cs = o.get_state()
    o2 = O.OracleStepper(m, p)
    o2.set_state(ph, cc, cl, cs)
    v = np.random.default_rng(9).standard_normal(2 * m.cells()) * 1e-3
    an = o2.jv(v, 0.1, 1)
    fd = o2.jv(v, 0.1, 0)
    n = m.cells()
    for rows in (slice(0, n), slice(n, 2 * n)):
        assert O.rel_l2(an[rows] - v[rows], fd[rows] - v[rows]) <= 1e-5
