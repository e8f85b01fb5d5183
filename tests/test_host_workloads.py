"""Host-side checks of the synthetic workloads (CPU): the random CALPHAD
draws keep both phases convex (unique KKS split), the seeded initial states
are deterministic and within range, the orientation fields are unit
vectors, and the integrator parameters carry CVODE's constants."""
import numpy as np
import pytest

from ampe_gb300 import abi, configs, initial


@pytest.mark.parametrize("seed", [1, 3, 7])
def test_random_rk_convex(seed):
    L = configs.random_rk(seed)
    c = np.linspace(0.01, 0.99, 99)
    for T in (1250.0, 1500.0, 1750.0):
        for p in range(2):
            f2 = configs.R_GAS * T / (c * (1 - c)) - 2 * L[p, 0] - 6 * L[p, 1] * (2 * c - 1)
            assert f2.min() > 0.0
    assert np.all(np.abs(L) <= 2.0e4)


def test_calphad3d_model():
    m = configs.calphad3d(32, seed=3, T_run=1500.0)
    assert m.dim == 3 and m.cells() == 32 ** 3
    assert m.thermo == abi.THERMO_CALPHAD and m.temp_mode == abi.TEMP_GRADIENT
    # T spans T_run - 25 .. T_run + 25 across the level
    t_lo = m.T0 + 0.5 * m.gradT * m.dx[0]
    t_hi = m.T0 + (32 - 0.5) * m.gradT * m.dx[0]
    assert abs(0.5 * (t_lo + t_hi) - 1500.0) < 1e-9
    assert abs((t_hi - t_lo) - 50.0 * 31.0 / 32.0) < 1e-9


def test_states_deterministic_and_in_range():
    a = initial.calphad3d_state(16, seed=2, nseeds=2, radius=4.5)
    b = initial.calphad3d_state(16, seed=2, nseeds=2, radius=4.5)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    phi, c = a
    assert phi.min() >= 0.0 and phi.max() <= 1.0
    assert c.min() >= 0.3 and c.max() <= 0.5


def test_polycrystal_state():
    phi, c, q = initial.polycrystal_state(24, ngrains=4, seed=1, channel=4.0)
    assert phi.shape == (24, 24, 24) and q.shape == (4, 24, 24, 24)
    assert np.allclose(np.linalg.norm(q, axis=0), 1.0)
    assert phi.min() >= 0.0 and phi.max() <= 1.0
    assert phi.max() > 0.9 and phi.min() < 0.1  # solid grains, liquid channels


def test_dendrite_state():
    phi, c, q = initial.dendrite2d_state(64, nseeds=4, radius=6.0, seed=3)
    assert phi.shape == (1, 64, 64) and q.shape == (2, 1, 64, 64)
    assert np.allclose(q[0] ** 2 + q[1] ** 2, 1.0)
    assert np.all(q[1] >= 0.0)  # angles in [0, pi)
    assert abs(c.mean() - 0.02) < 1e-3


def test_dendrite_undercooling():
    m = configs.dendrite2d(64, undercooling=0.55)
    c0, Tm, ml, k = 0.02, 933.0, -260.0, 0.14
    T_L = Tm + ml * c0
    dT0 = abs(ml) * c0 * (1 - k) / k
    assert abs(m.T0 - (T_L - 0.55 * dT0)) < 1e-9
    assert m.flux_type == abi.FLUX_ANISOTROPIC and m.aniso_k == 4


def test_step_params_cvode_constants():
    p = configs.step_params(atol=1e-6)
    assert p.max_newton == 3 and p.max_krylov == 5
    assert abs(p.newton_coef - 0.2) < 1e-15 and abs(p.lin_coef - 0.05) < 1e-15
    assert abs(p.rtol - 1e-8) < 1e-20
