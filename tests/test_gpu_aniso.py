"""2D anisotropic phase flux (anisotropic_gradient_flux, 2d/quatrhs.m4:
154-256) inside the implicit stepper: the dendrite workload (four-fold
anisotropy delta = 0.02, dilute KKS, seeds with their own orientation
angles) against the CPU oracle.  Bars: FP64 steps relative L2 <= 1e-10 with
identical solver counts; the mixed path's analytic FP32 Jacobian-vector
product (linearised anisotropic flux) within 1e-3 of the oracle's FP64
finite-difference product where the flux is differentiable at the FD scale
(interface region), within 5e-2 on the whole level, composition rows within
1e-5 of the oracle's analytic product; mixed steps within 2e-6 of the FP64
oracle.  3D cubic anisotropy (anisotropic_gradient_flux, 3d/quatrhs.m4:
180-355) with a static two-grain orientation field: FP64 steps as above,
the mixed path (FP32 flux, Jacobian by forward-mode differentiation) within
2e-6 of the oracle and its phase-row product within 1e-3 of the FD product
around the interfaces; an evolving orientation is refused by the mixed
path."""
import numpy as np
import pytest

import oracle as O
from ampe_gb300 import configs, initial
from ampe_gb300.stepper import ImplicitStepper

pytestmark = pytest.mark.gpu


def case(n=64):
    m = configs.dendrite2d(n)
    phi, c, q = initial.dendrite2d_state(n, nseeds=3, radius=8, seed=2)
    return m, phi, c, q


@pytest.mark.parametrize("precond", [0, 1, 2])
def test_fp64_steps(cuda, precond):
    m, phi, c, q = case()
    p = configs.step_params(dt=0.1, precond=precond, mg_levels=3, atol=1e-6)
    o = O.OracleStepper(m, p)
    o.set_state(phi, c)
    o.set_orientation(q)
    rc, so = o.advance(4)
    assert rc == 0
    g = ImplicitStepper(m, p)
    g.set_state(phi, c)
    g.set_orientation(q)
    sg = g.advance(4)
    for k in ("steps", "newton_iters", "gmres_iters", "rhs_evals", "precond_solves",
              "fac_cycles"):
        assert sg[k] == so[k], (k, sg[k], so[k])
    for a, b in zip(g.get_state(), o.get_state()):
        assert O.rel_l2(a, b) <= 1e-10


def test_orientation_matters(cuda):
    """Rotating the orientation field changes the solution (the flux reads it)."""
    m, phi, c, q = case()
    p = configs.step_params(dt=0.1, precond=2, mg_levels=3, atol=1e-6)
    out = []
    for qq in (q, np.stack([np.cos(0.3 + np.arccos(q[0])), np.sin(0.3 + np.arccos(q[0]))])):
        g = ImplicitStepper(m, p)
        g.set_state(phi, c)
        g.set_orientation(np.ascontiguousarray(qq))
        g.advance(3)
        out.append(g.get_state()[0])
    assert O.rel_l2(out[0], out[1]) > 1e-6


def test_mixed_jv_vs_fd(cuda):
    m, phi, c, q = case()
    p64 = configs.step_params(precond=2, mg_levels=3, atol=1e-6)
    o = O.OracleStepper(m, p64)
    o.set_state(phi, c)
    o.set_orientation(q)
    o.advance(2)
    ph, cc, cl, cs = o.get_state()
    o.set_state(ph, cc, cl, cs)
    o.set_orientation(q)
    pm = configs.step_params(precond=2, mg_levels=3, atol=1e-6, precision=1)
    gm = ImplicitStepper(m, pm)
    gm.set_state(ph, cc, cl, cs)
    gm.set_orientation(q)
    v = np.random.default_rng(21).standard_normal(2 * m.cells()) * 1e-3
    fd = o.jv(v, 0.1, 0)
    an = gm.jv(v, 0.1)
    N = m.cells()
    # composition rows: the anisotropy does not enter; against the oracle's
    # analytic product (the FD product carries O(sigma v / c) truncation from
    # the logarithms of the dilute model at c ~ 0.003)
    ex = o.jv(v, 0.1, 1)
    s = slice(N, 2 * N)
    assert O.rel_l2(an[s] - v[s], ex[s] - v[s]) <= 1e-5
    # phase rows.  The flux is homogeneous of degree one in grad phi with a
    # direction-dependent eps(theta): where |grad phi| is far below the FD
    # perturbation (sigma v ~ atol) the one-sided FD product samples F along
    # the perturbation's direction, the linearisation along grad phi's, and the
    # two differ at the O(nu k^2) level of the anisotropy.  Around the
    # interfaces (|grad phi| well above the perturbation on the whole stencil)
    # both are the derivative and must agree.
    p2 = ph[0]
    gx = 0.5 * (np.roll(p2, -1, 1) - np.roll(p2, 1, 1))
    gy = 0.5 * (np.roll(p2, -1, 0) - np.roll(p2, 1, 0))
    gm2 = np.hypot(gx, gy)
    lo = gm2.copy()
    for sy in (-1, 0, 1):
        for sx in (-1, 0, 1):
            lo = np.minimum(lo, np.roll(np.roll(gm2, sy, 0), sx, 1))
    mask = (lo > 1e-3).ravel()
    assert mask.sum() > 100
    da, df = (an[:N] - v[:N]), (fd[:N] - v[:N])
    err_if = O.rel_l2(da[mask], df[mask])
    err_all = O.rel_l2(da, df)
    print("aniso Jv phase rows: interface %.2e, whole level %.2e" % (err_if, err_all))
    assert err_if <= 1e-3
    assert err_all <= 5e-2


def test_mixed_steps(cuda):
    m, phi, c, q = case()
    p64 = configs.step_params(dt=0.1, precond=2, mg_levels=3, atol=1e-6)
    o = O.OracleStepper(m, p64)
    o.set_state(phi, c)
    o.set_orientation(q)
    rc, so = o.advance(6)
    assert rc == 0
    pm = configs.step_params(dt=0.1, precond=2, mg_levels=3, atol=1e-6, precision=1)
    g = ImplicitStepper(m, pm)
    g.set_state(phi, c)
    g.set_orientation(q)
    sg = g.advance(6)
    assert sg["steps"] == 6 and sg["kks_fail"] == 0
    errs = [O.rel_l2(a, b) for a, b in zip(g.get_state()[:2], o.get_state()[:2])]
    print("mixed dendrite vs FP64 oracle rel L2 (phi, c):", errs, sg)
    assert max(errs) <= 2e-6


def case3d(n=20):
    """3D CALPHAD with the cubic anisotropic flux (eps4 = 0.05), two seeds and
    a static orientation field of two grains split along x."""
    from ampe_gb300 import abi

    m = configs.calphad3d(n, seed=3, T_run=1500.0)
    m.flux_type = abi.FLUX_ANISOTROPIC
    m.qlen = 4
    m.aniso_eps = 0.05
    phi, c = initial.calphad3d_state(n, seed=2, nseeds=2, radius=5.0)
    rng = np.random.default_rng(13)
    qa = rng.standard_normal(4)
    qb = rng.standard_normal(4)
    qa /= np.linalg.norm(qa)
    qb /= np.linalg.norm(qb)
    x = np.arange(n)
    q = np.where((x < n // 2)[None, None, None, :], qa[:, None, None, None],
                 qb[:, None, None, None]) * np.ones((4, n, n, n))
    return m, phi, c, np.ascontiguousarray(q)


def test_fp64_steps_3d(cuda):
    m, phi, c, q = case3d()
    p = configs.step_params(dt=0.1, precond=2, mg_levels=3, atol=1e-6)
    o = O.OracleStepper(m, p)
    o.set_state(phi, c)
    o.set_orientation(q)
    rc, so = o.advance(3)
    assert rc == 0
    g = ImplicitStepper(m, p)
    g.set_state(phi, c)
    g.set_orientation(q)
    sg = g.advance(3)
    for k in ("steps", "newton_iters", "gmres_iters", "rhs_evals", "precond_solves"):
        assert sg[k] == so[k], (k, sg[k], so[k])
    for a, b in zip(g.get_state(), o.get_state()):
        assert O.rel_l2(a, b) <= 1e-10


def test_mixed_3d_steps_and_jv(cuda):
    """The mixed path with the FP32 3D anisotropic flux and its forward-mode
    Jacobian: steps within 2e-6 of the FP64 oracle; the Jacobian-vector
    product's phase rows within 1e-3 of the oracle's FP64 finite-difference
    product around the interfaces."""
    m, phi, c, q = case3d()
    p64 = configs.step_params(dt=0.1, precond=2, mg_levels=3, atol=1e-6)
    o = O.OracleStepper(m, p64)
    o.set_state(phi, c)
    o.set_orientation(q)
    rc, so = o.advance(4)
    assert rc == 0
    pm = configs.step_params(dt=0.1, precond=2, mg_levels=3, atol=1e-6, precision=1)
    g = ImplicitStepper(m, pm)
    g.set_state(phi, c)
    g.set_orientation(q)
    sg = g.advance(4)
    assert sg["steps"] == 4 and sg["kks_fail"] == 0
    errs = [O.rel_l2(a, b) for a, b in zip(g.get_state()[:2], o.get_state()[:2])]
    print("mixed 3D aniso vs FP64 oracle rel L2 (phi, c):", errs, sg)
    assert max(errs) <= 2e-6
    ph, cc, cl, cs = o.get_state()
    o.set_state(ph, cc, cl, cs)
    o.set_orientation(q)
    g.set_state(ph, cc, cl, cs)
    v = np.random.default_rng(22).standard_normal(2 * m.cells()) * 1e-3
    fd = o.jv(v, 0.1, 0)
    an = g.jv(v, 0.1)
    N = m.cells()
    p3 = ph
    gr = np.sqrt(sum((0.5 * (np.roll(p3, -1, a) - np.roll(p3, 1, a))) ** 2 for a in range(3)))
    lo = gr.copy()
    for a in range(3):
        for sh in (-1, 1):
            lo = np.minimum(lo, np.roll(gr, sh, a))
    mask = (lo > 1e-3).ravel()
    assert mask.sum() > 100
    err_if = O.rel_l2(an[:N][mask] - v[:N][mask], fd[:N][mask] - v[:N][mask])
    print("3D aniso Jv phase rows, interface: %.2e" % err_if)
    assert err_if <= 1e-3


def test_mixed_aniso_evolving_orientation_rejected(cuda):
    m = configs.calphad3d(16, seed=3, T_run=1500.0)
    from ampe_gb300 import abi
    m.flux_type = abi.FLUX_ANISOTROPIC
    m.qlen = 4
    m.aniso_eps = 0.05
    m.evolve_quat = 1
    from ampe_gb300._native import AmpeError
    with pytest.raises(AmpeError):
        ImplicitStepper(m, configs.step_params(precision=1))
