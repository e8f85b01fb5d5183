"""Model and integrator parameter sets for the benchmark workloads.

Workloads (seeded, synthetic; the reference ships no data sets for them):

* ``dilute2d``   -- 2D phi + c, KKS dilute binary (k=0.14, liquidus slope
  -2.6 K/at% = -260 K per mole fraction, Tm = 933 K as in the reference's
  AlCu deck tests/AlCu/*.input, T = 900 K), isotropic 9-point flux,
  eps = 1, M_phi = 1, D_L = 1, D_S = 1e-4, dx = 1, periodic.
* ``calphad3d``  -- 3D phi + c, binary CALPHAD regular solution with two
  Redlich-Kister coefficients per phase drawn in [-2e4, 2e4] J/mol (pure
  species energies zero; draws rejected until each phase's free energy is
  convex on [0.01, 0.99] so the KKS split is unique), T = T_run + a linear
  50 K gradient along x, simple 7-point flux.

Unit conventions: lengths in cells (dx = 1), time in model units.  The
energy density scale 1e-6/Vm is chosen so that RT 1e-6/Vm ~ 0.1, the order
of the double-well height; the reference takes it from molar_volume.
"""
import numpy as np

from . import abi

R_GAS = 8.314472


def _blank_model(dim, n, ng=1):
    m = abi.Model()
    m.dim = dim
    m.n[0], m.n[1] = n[0], n[1]
    m.n[2] = n[2] if dim == 3 else 1
    m.ng = ng
    for d in range(3):
        m.dx[d] = 1.0
    m.flux_type = abi.FLUX_SIMPLE
    m.epsilon_phi = 1.0
    m.aniso_eps = 0.0
    m.aniso_k = 4
    m.qlen = 2
    m.phase_well_scale = 1.0 / 72.0  # interface width 3 cells: eps/sqrt(8 w)
    m.phase_mobility = 1.0
    m.well_type = b"d"
    m.energy_interp = b"p"
    m.conc_interp = b"p"
    m.diff_interp = b"p"
    m.avg_type = b"a"
    m.orient_interp1 = b"p"
    m.orient_interp2 = b"p"
    m.with_orient = 0
    m.conc_mobility = 1.0
    m.D_liquid = 1.0
    m.D_solid = 1.0e-4
    m.Q_liquid = 0.0
    m.Q_solid = 0.0
    m.newton_max_its = 50
    m.newton_tol = 1.0e-12
    m.temp_mode = abi.TEMP_CONSTANT
    m.evolve_quat = 0
    m.quat_mobility = 1.0
    m.min_quat_mobility = 1.0e-6
    m.quat_grad_floor = 1.0e-2
    m.quat_floor_type = b"s"
    m.quat_mobility_type = b"p"
    return m


def dilute2d(n=256, T=900.0):
    m = _blank_model(2, (n, n))
    m.flux_type = abi.FLUX_ISOTROPIC
    m.thermo = abi.THERMO_DILUTE
    m.dilute_Tm = 933.0
    m.dilute_m = -260.0
    m.dilute_k = 0.14
    m.conc_interp = b"l"
    ivm = 0.1 / (R_GAS * T)
    m.inv_molar_volume[0] = ivm
    m.inv_molar_volume[1] = ivm
    m.T0 = T
    m.temp_mode = abi.TEMP_CONSTANT
    return m


def dendrite2d(n=2048, undercooling=0.55, delta=0.02):
    """dilute2d with the 2D four-fold anisotropic flux (delta = 0.02, qlen 2)
    at the temperature of a dimensionless undercooling
    (T_L(c0) - T) / dT0 = undercooling, T_L(c0) = Tm + m c0 with c0 = 0.02 and
    the freezing range dT0 = |m| c0 (1 - k) / k."""
    c0, Tm, mliq, k = 0.02, 933.0, -260.0, 0.14
    T_L = Tm + mliq * c0
    dT0 = abs(mliq) * c0 * (1.0 - k) / k
    T = T_L - undercooling * dT0
    m = dilute2d(n, T=T)
    m.flux_type = abi.FLUX_ANISOTROPIC
    m.aniso_eps = delta
    m.aniso_k = 4
    m.qlen = 2
    return m


def random_rk(seed, T_check=(1250.0, 1750.0), lim=2.0e4):
    """Two Redlich-Kister coefficients (L0, L1) per phase, convex draws."""
    rng = np.random.default_rng(seed)
    c = np.linspace(0.01, 0.99, 197)
    while True:
        L = rng.uniform(-lim, lim, size=(2, 2))
        ok = True
        for T in T_check:
            for p in range(2):
                f2 = R_GAS * T / (c * (1 - c)) - 2 * L[p, 0] - 6 * L[p, 1] * (2 * c - 1)
                if f2.min() < 0.25 * R_GAS * T:
                    ok = False
        if ok:
            return L


def calphad3d(n=256, seed=3, T_run=None, gradT_total=50.0):
    m = _blank_model(3, (n, n, n))
    m.thermo = abi.THERMO_CALPHAD
    rng = np.random.default_rng(seed + 1000)
    if T_run is None:
        T_run = float(rng.uniform(1300.0, 1700.0))
    L = random_rk(seed)
    for p in range(2):
        m.L[p][0][0] = L[p, 0]
        m.L[p][1][0] = L[p, 1]
    # pure species energies zero (g[*][*].nseg = 0)
    ivm = 0.1 / (R_GAS * T_run)
    m.inv_molar_volume[0] = ivm
    m.inv_molar_volume[1] = ivm
    m.T0 = T_run - 0.5 * gradT_total
    m.gradT = gradT_total / (n * m.dx[0])
    m.temp_mode = abi.TEMP_GRADIENT
    return m


def polycrystal3d(n=128, seed=3, T=1500.0):
    """phi + c + quaternion polycrystal: CALPHAD as calphad3d at constant T,
    quaternion mobility with the 1/|grad q| regularisation (floor 1e-2)."""
    m = calphad3d(n, seed=seed, T_run=T, gradT_total=0.0)
    m.temp_mode = abi.TEMP_CONSTANT
    m.T0 = T
    m.gradT = 0.0
    m.with_orient = 1
    m.evolve_quat = 1
    m.epsilon_q = 0.5
    m.misorientation_factor = 2.0e-5  # 2 H: 2H T |grad q| ~ w at a boundary
    m.quat_mobility = 1.0
    m.min_quat_mobility = 1.0e-6
    m.quat_grad_floor = 1.0e-2
    m.quat_floor_type = b"s"
    return m


def step_params(dt=0.1, precond=2, precision=0, surrogate=0, mg_levels=5,
                atol=3.0e-4):
    p = abi.StepParams()
    p.dt = dt
    p.max_order = 2
    p.atol = atol
    p.rtol = atol * 1.0e-2  # QuatIntegrator.cc:287
    p.max_newton = 3  # CVODE maxcor
    p.newton_coef = 0.2  # CVODE tq[4] for BDF1 (nlscoef 0.1 / tq[2] 0.5)
    p.max_krylov = 5  # QuatIntegrator.cc:297
    p.lin_coef = 0.05  # CVODE eplifac
    p.precond = precond
    p.fac_max_cycles = 10  # FACPreconditioner.cc:83
    p.rb_sweeps = 5  # tests/KKScomposition/3d.input:84-86
    p.rb_tol = -1.0
    p.mg_levels = mg_levels
    p.mg_pre = 1  # FACPreconditioner.cc:98-106
    p.mg_post = 1
    p.mg_coarse_sweeps = 4
    p.precision = precision
    p.surrogate = surrogate
    p.max_retries = 3
    return p
