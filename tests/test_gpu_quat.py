"""Quaternion orientation path on the GPU against the CPU oracle: the leaf
kernels (|grad q|, M_q, face coefficients for each floor type, -M_q
div(fc grad q)), the fused phase RHS with the orientation term, and full
BDF steps of phi + c + q (FP64).  Parity bar: leaf kernels relative L2
<= 1e-12; steps <= 1e-10 per field with identical solver counts."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from ampe_gb300 import abi, configs, initial
from ampe_gb300.stepper import ImplicitStepper

pytestmark = pytest.mark.gpu
TOL = 1e-12

_KEEP = []


@pytest.fixture(autouse=True)
def _keep_alive():
    yield
    _KEEP.clear()


def dev(a):
    import torch

    t = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()
    _KEEP.append(t)
    return t


def host(t):
    import torch

    torch.cuda.synchronize()
    return t.cpu().numpy()


def P(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def quat_model(dim, floor_type=b"s", n=12):
    if dim == 3:
        m = configs.polycrystal3d(n, seed=3, T=1500.0)
    else:
        m = configs.polycrystal3d(n, seed=3, T=1500.0)
        m.dim = 2
        m.n[2] = 1
    m.quat_floor_type = floor_type
    return m


def rand_quat_ghosted(m, rng, smooth=True):
    shp = m.interior_shape()
    q = rng.standard_normal((4,) + tuple(shp))
    if smooth:  # a few grains plus noise so |grad q| spans the floor
        q = np.round(q) + 0.05 * rng.standard_normal(q.shape)
    q /= np.linalg.norm(q, axis=0, keepdims=True)
    return np.concatenate([O.ghosted(m, q[c]).ravel() for c in range(4)])


def nfaces(m):
    n0, n1, n2 = m.n[0], m.n[1], m.n[2] if m.dim == 3 else 1
    return ((n0 + 1) * n1 * n2, n0 * (n1 + 1) * n2, n0 * n1 * (n2 + 1) if m.dim == 3 else 1)


@pytest.mark.parametrize("dim", [2, 3])
def test_grad_modulus_and_mobility(cuda, orc, dim):
    m = quat_model(dim)
    rng = np.random.default_rng(11)
    q = rand_quat_ghosted(m, rng)
    N = m.cells()
    o = np.empty(N)
    orc.orc_quat_grad_modulus(C.byref(m), q.ctypes.data, o.ctypes.data)
    gq = dev(q)
    go = dev(np.zeros(N))
    assert cuda.lib.ampe_quat_grad_modulus(C.byref(m), P(gq), P(go), None) == 0
    assert O.rel_l2(host(go), o) <= TOL
    phi = O.ghosted(m, rng.uniform(-0.1, 1.1, size=m.interior_shape()))
    mo = np.zeros_like(phi)
    orc.orc_quat_mobility(C.byref(m), phi.ctypes.data, mo.ctypes.data)
    gm = dev(np.zeros_like(phi))
    assert cuda.lib.ampe_quat_mobility(C.byref(m), P(dev(phi)), P(gm), None) == 0
    assert O.rel_l2(host(gm), mo) <= TOL


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("floor_type", [b"m", b"s", b"t"])
def test_face_coef_and_rhs(cuda, orc, dim, floor_type):
    m = quat_model(dim, floor_type)
    rng = np.random.default_rng(5)
    q = rand_quat_ghosted(m, rng)
    phi = O.ghosted(m, rng.uniform(0.0, 1.0, size=m.interior_shape()))
    nf = nfaces(m)
    fo = [np.zeros(k) for k in nf]
    orc.orc_quat_face_coef(C.byref(m), phi.ctypes.data, None, q.ctypes.data,
                           *[f.ctypes.data for f in fo])
    fg = [dev(np.zeros(k)) for k in nf]
    gq, gphi = dev(q), dev(phi)
    assert cuda.lib.ampe_quat_face_coef(C.byref(m), P(gphi), None, P(gq),
                                        *[P(f) for f in fg], None) == 0
    for d in range(dim):
        assert O.rel_l2(host(fg[d]), fo[d]) <= TOL
    mq = np.zeros_like(phi)
    orc.orc_quat_mobility(C.byref(m), phi.ctypes.data, mq.ctypes.data)
    ro = np.empty(4 * m.cells())
    orc.orc_quat_rhs(C.byref(m), *[f.ctypes.data for f in fo], mq.ctypes.data,
                     q.ctypes.data, ro.ctypes.data)
    rg = dev(np.zeros(4 * m.cells()))
    assert cuda.lib.ampe_quat_rhs(C.byref(m), *[P(f) for f in fg], P(dev(mq)), P(gq),
                                  P(rg), None) == 0
    assert O.rel_l2(host(rg), ro) <= TOL


def test_face_coef_rejects_bad_floor(cuda):
    m = quat_model(3)
    m.quat_grad_floor = 0.0
    x = dev(np.zeros(4 * (m.n[0] + 2) ** 3))
    assert cuda.lib.ampe_quat_face_coef(C.byref(m), P(x), None, P(x), P(x), P(x), P(x),
                                        None) == abi.AMPE_ERR_INVALID


def poly_case(n=16, ngrains=4):
    m = configs.polycrystal3d(n, seed=3, T=1500.0)
    phi, c, q = initial.polycrystal_state(n, ngrains=ngrains, seed=1, channel=4.0)
    return m, phi, c, q


def test_eval_rhs_full_parity(cuda):
    m, phi, c, q = poly_case()
    p = configs.step_params(precond=2, mg_levels=3, atol=1e-6)
    o = O.OracleStepper(m, p)
    o.set_state(phi, c)
    o.set_quat(q)
    g = ImplicitStepper(m, p)
    g.set_state(phi, c)
    g.set_quat(q)
    assert g.size() == 6 * m.cells()
    fo = o.eval_rhs_full()
    fg = g.eval_rhs_full()
    N = m.cells()
    for b in range(6):
        assert O.rel_l2(fg[b * N:(b + 1) * N], fo[b * N:(b + 1) * N]) <= 1e-11, b
    # the orientation term is live: q moves at the grain boundaries
    assert np.abs(fg[2 * N:]).max() > 0.0


@pytest.mark.parametrize("precond", [0, 1, 2])
def test_steps_parity(cuda, precond):
    m, phi, c, q = poly_case()
    p = configs.step_params(dt=0.1, precond=precond, mg_levels=3, atol=1e-6)
    nsteps = 3
    o = O.OracleStepper(m, p)
    o.set_state(phi, c)
    o.set_quat(q)
    rc, so = o.advance(nsteps)
    assert rc == 0
    g = ImplicitStepper(m, p)
    g.set_state(phi, c)
    g.set_quat(q)
    sg = g.advance(nsteps)
    for k in ("steps", "newton_iters", "gmres_iters", "rhs_evals", "precond_solves",
              "fac_cycles"):
        assert sg[k] == so[k], (k, sg[k], so[k])
    for a, b in zip(g.get_state(), o.get_state()):
        assert O.rel_l2(a, b) <= 1e-10
    qg, qo = g.get_quat(), o.get_quat()
    assert O.rel_l2(qg, qo) <= 1e-10
    # accepted states are unit quaternions
    assert np.abs(np.linalg.norm(qg, axis=0) - 1.0).max() < 1e-12
    assert np.abs(qg - q).max() > 1e-6  # and the orientation evolved


def test_fd_jv_parity(cuda):
    m, phi, c, q = poly_case()
    p = configs.step_params(precond=1, atol=1e-6)
    o = O.OracleStepper(m, p)
    o.set_state(phi, c)
    o.set_quat(q)
    g = ImplicitStepper(m, p)
    g.set_state(phi, c)
    g.set_quat(q)
    v = np.random.default_rng(4).standard_normal(6 * m.cells()) * 1e-3
    jo = o.jv(v, 0.05, analytic=False)
    jg = g.jv(v, 0.05)
    assert O.rel_l2(jg, jo) <= 1e-9


def test_mixed_jv_vs_fd(cuda):
    """FP32 analytic product (q rows, orientation term of the phase row,
    lagged gradients) against the oracle's FP64 finite-difference product."""
    m, phi, c, q = poly_case()
    p64 = configs.step_params(precond=2, mg_levels=3, atol=1e-6)
    o = O.OracleStepper(m, p64)
    o.set_state(phi, c)
    o.set_quat(q)
    o.advance(2)
    ph, cc, cl, cs = o.get_state()
    qq = o.get_quat()
    o.set_state(ph, cc, cl, cs)
    o.set_quat(qq)
    pm = configs.step_params(precond=2, mg_levels=3, atol=1e-6, precision=1)
    gm = ImplicitStepper(m, pm)
    gm.set_state(ph, cc, cl, cs)
    gm.set_quat(qq)
    v = np.random.default_rng(12).standard_normal(6 * m.cells()) * 1e-3
    fd = o.jv(v, 0.1, 0)
    an = gm.jv(v, 0.1)
    N = m.cells()
    for b in range(6):
        s = slice(b * N, (b + 1) * N)
        err = O.rel_l2(an[s] - v[s], fd[s] - v[s])
        assert err <= 1e-4, (b, err)


def test_mixed_steps_vs_oracle(cuda):
    m, phi, c, q = poly_case()
    nsteps = 4
    p64 = configs.step_params(dt=0.1, precond=2, mg_levels=3, atol=1e-6)
    o = O.OracleStepper(m, p64)
    o.set_state(phi, c)
    o.set_quat(q)
    rc, so = o.advance(nsteps)
    assert rc == 0
    pm = configs.step_params(dt=0.1, precond=2, mg_levels=3, atol=1e-6, precision=1)
    g = ImplicitStepper(m, pm)
    g.set_state(phi, c)
    g.set_quat(q)
    sg = g.advance(nsteps)
    assert sg["steps"] == nsteps and sg["kks_fail"] == 0
    errs = [O.rel_l2(a, b) for a, b in zip(g.get_state()[:2], o.get_state()[:2])]
    errs.append(O.rel_l2(g.get_quat(), o.get_quat()))
    print("mixed polycrystal vs FP64 oracle rel L2 (phi, c, q):", errs, sg)
    assert max(errs) <= 2e-6
    assert np.abs(np.linalg.norm(g.get_quat(), axis=0) - 1.0).max() < 1e-12
